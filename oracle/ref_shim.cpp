/*
 * ref_shim.cpp -- TEST INFRASTRUCTURE.  Builds the reference's own CPU path for
 * the pair kernels into oracle/_ref/libmfref.so (see oracle/Makefile), so the
 * oracle restatement and the golden fixtures can be checked against the
 * reference itself.  Compiled only where the reference sources are present.
 *
 * Each entry point runs fmmtl::direct (fmmtl_minimum/fmmtl/Direct.hpp:18-28,
 * dispatching to S2T.hpp:57-79) over the reference kernels
 *   DipoleBKernel        fmmtl_minimum/kernel/Dipole_B.kern:13-134
 *   DipoleHessianKernel  fmmtl_minimum/kernel/Dipole_hessian.kern:19-278
 * in the reference's FP32 (_K_real_ = float), split over targets with OpenMP.
 * Arrays are AoS float [n][3]; tensors are [n][9] glm column-major.
 */
#include "kernel/Dipole_B.kern"
#include "kernel/Dipole_hessian.kern"
#include "fmmtl/Direct.hpp"

#include <cstdint>
#include <vector>

typedef Vec<3, float> V3;

extern "C" int ref_field(int64_t nt, const float* tpos, int64_t ns, const float* spos,
                         const float* smom, float h, float* out) {
  const V3* S = reinterpret_cast<const V3*>(spos);
  const V3* C = reinterpret_cast<const V3*>(smom);
  const V3* T = reinterpret_cast<const V3*>(tpos);
  V3* R = reinterpret_cast<V3*>(out);
  DipoleBKernel K(h);
#pragma omp parallel for schedule(dynamic, 16)
  for (int64_t i = 0; i < nt; ++i) {
    R[i] = V3(0, 0, 0);
    fmmtl::direct(K, S, S + ns, C, T + i, T + i + 1, R + i);
  }
  return 0;
}

extern "C" int ref_tensor(int64_t nt, const float* tpos, int64_t ns, const float* spos,
                          const float* smom, float h, float* out9) {
  const V3* S = reinterpret_cast<const V3*>(spos);
  const V3* C = reinterpret_cast<const V3*>(smom);
  const V3* T = reinterpret_cast<const V3*>(tpos);
  DipoleHessianKernel K(h);
#pragma omp parallel for schedule(dynamic, 16)
  for (int64_t i = 0; i < nt; ++i) {
    glm::mat3 acc(0.0f);
    fmmtl::direct(K, S, S + ns, C, T + i, T + i + 1, &acc);
    for (int c = 0; c < 3; ++c)
      for (int r = 0; r < 3; ++r) out9[9 * i + 3 * c + r] = acc[c][r];
  }
  return 0;
}

extern "C" int ref_abi_version(void) { return 1; }
