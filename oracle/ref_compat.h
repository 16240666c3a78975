/*
 * ref_compat.h -- TEST INFRASTRUCTURE.  Force-included when oracle/Makefile
 * compiles the reference's own FMMTL kernels into oracle/_ref.
 *
 * The reference was written against Thrust 1.8, which provided
 * thrust::detail::enable_if_convertible (used by fmmtl/meta/range.hpp:92-93).
 * The CUDA 13 CCCL no longer ships it; this supplies the same trait so the
 * unmodified reference headers compile.
 */
#pragma once
#include <type_traits>
#include <thrust/detail/type_traits.h>
namespace thrust {
namespace detail {
template <typename From, typename To, typename R = void>
struct enable_if_convertible : std::enable_if<std::is_convertible<From, To>::value, R> {};
}  // namespace detail
}  // namespace thrust
