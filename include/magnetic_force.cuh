// magnetic_force.cuh -- drop-in C++ surface of the reference's solver class
//   Libo::cuda_magnet_cgOptimizer   (magnetic_solver/magnetic_force.cuh:36-174)
// implemented header-only on the C ABI of libmfgb.so (include/mf.h).
//
// A caller written against the reference (e.g. magnetic_solver/main.cu)
// compiles unchanged with this directory first on the include path and links
// libmfgb.so instead of magnetic_force.cu + FMMTL.  Kept: the CtorParam and
// setHextParams types, the constructor, Resize, setTargetpos, setHext, solve,
// evaluate_fitted_near_foece, clear, export_data, export_force, the knobs
// tolerance / max_iteration / naive / crit_size, and the result members
// (xyz, M, total_B_over_mu0, Hext, magnetic_bodyforce, dHextdx/dy/dz) as
// device SoA views with dev_x / dev_y / dev_z / np like cuda_abstract_vector.
// The solver's internal steps (start, step_iteration, G, D, calc_alpha, ...)
// are not exposed: they run on the device inside solve().
//
// Errors: the reference reports none; here a failing call throws
// std::runtime_error carrying the library's message.
#pragma once
#ifndef LIBO_MAGNETIC_FORCE_SOLVER
#define LIBO_MAGNETIC_FORCE_SOLVER

#include <cuda_runtime.h>
#include <vector_types.h>

#include <cstddef>
#include <stdexcept>
#include <string>
#include <vector>

#include "mf.h"

namespace Libo {

// Non-owning device SoA view with the reference's member names
// (magnetic_solver/cuda_abstract_vector.cuh:238-242).
template <typename T>
class cuda_abstract_vector {
 public:
  cudaError_t cudaStatus = cudaSuccess;
  size_t np = 0;
  T* dev_x = nullptr;
  T* dev_y = nullptr;
  T* dev_z = nullptr;
  typedef T value_type;
  mf_solver* owner = nullptr;  // the solver publishing this quantity
  int quantity = 0;            // its mf_quantity

  // Copies the three components to host memory (through the library, so the
  // caller does not need to link the CUDA runtime itself).
  void export_data(T* host_x, T* host_y, T* host_z) const {
    std::vector<float> soa(3 * np);
    mf_status s = mf_get(owner, quantity, soa.data(), MF_LAYOUT_SOA, MF_HOST);
    if (s != MF_OK) throw std::runtime_error(std::string(mf_status_string(s)) + ": " + mf_last_error());
    for (size_t i = 0; i < np; ++i) {
      host_x[i] = T(soa[i]);
      host_y[i] = T(soa[np + i]);
      host_z[i] = T(soa[2 * np + i]);
    }
  }
  void export_data(std::vector<T>& host_x, std::vector<T>& host_y, std::vector<T>& host_z) const {
    host_x.resize(np);
    host_y.resize(np);
    host_z.resize(np);
    export_data(host_x.data(), host_y.data(), host_z.data());
  }
};

class cuda_magnet_cgOptimizer {
 public:
  struct CtorParam {
    CtorParam(size_t _num_particles, float _h, float _ext_mag_h, float _volume, float _chi,
              float* _const_ext_field, const std::vector<float3>& _ext_source_pos,
              const std::vector<float3>& _ext_source_M, const std::vector<float3>& _target_pos)
        : num_particles(_num_particles), h(_h), ext_mag_h(_ext_mag_h), volume(_volume), chi(_chi),
          ext_source_pos(_ext_source_pos), ext_source_M(_ext_source_M), target_pos(_target_pos) {
      const_ext_field[0] = _const_ext_field[0];
      const_ext_field[1] = _const_ext_field[1];
      const_ext_field[2] = _const_ext_field[2];
    }
    CtorParam(size_t _num_particles, float _h, float _ext_mag_h, float _volume, float _chi,
              float3 _const_ext_field, const std::vector<float3>&& _ext_source_pos,
              const std::vector<float3>&& _ext_source_M, const std::vector<float3>& _target_pos)
        : num_particles(_num_particles), h(_h), ext_mag_h(_ext_mag_h), volume(_volume), chi(_chi),
          ext_source_pos(_ext_source_pos), ext_source_M(_ext_source_M), target_pos(_target_pos) {
      const_ext_field[0] = _const_ext_field.x;
      const_ext_field[1] = _const_ext_field.y;
      const_ext_field[2] = _const_ext_field.z;
    }
    size_t num_particles;
    float h;
    float ext_mag_h;
    float volume;
    float chi;
    float const_ext_field[3];
    std::vector<float3> ext_source_pos;
    std::vector<float3> ext_source_M;
    std::vector<float3> target_pos;
  };

  struct setHextParams {
    float const_ext_field[3];
    std::vector<float3> ext_source_pos;
    std::vector<float3> ext_source_M;
    float ext_mag_h;
  };

  explicit cuda_magnet_cgOptimizer(const CtorParam& p, int device = 0) {
    if (p.target_pos.size() != p.num_particles) throw std::runtime_error("target_pos size != num_particles");
    mf_params q{};
    q.num_particles = int64_t(p.num_particles);
    q.h = p.h;
    q.ext_mag_h = p.ext_mag_h;
    q.volume = p.volume;
    q.chi = p.chi;
    for (int k = 0; k < 3; ++k) q.const_ext_field[k] = p.const_ext_field[k];
    q.target_pos = reinterpret_cast<const float*>(p.target_pos.data());
    q.n_ext = int64_t(p.ext_source_pos.size());
    q.ext_source_pos = q.n_ext ? reinterpret_cast<const float*>(p.ext_source_pos.data()) : nullptr;
    q.ext_source_M = q.n_ext ? reinterpret_cast<const float*>(p.ext_source_M.data()) : nullptr;
    q.precision = MF_FP32;
    q.device = device;
    check(mf_create(&q, &handle_));
    chi = p.chi;
    h = p.h;
    volume = p.volume;
    refresh();
  }
  ~cuda_magnet_cgOptimizer() { mf_destroy(handle_); }
  cuda_magnet_cgOptimizer(const cuda_magnet_cgOptimizer&) = delete;
  cuda_magnet_cgOptimizer& operator=(const cuda_magnet_cgOptimizer&) = delete;

  // Methods (magnetic_force.cuh:86-114) ---------------------------------------
  void Resize(size_t _np) {
    if (_np == np) return;
    // A resize without new positions keeps the first min(old, new) positions
    // and pads with copies of the last one until setTargetpos supplies them.
    std::vector<float> xyz_host(3 * np);
    check(mf_get(handle_, MF_Q_POSITIONS, xyz_host.data(), MF_LAYOUT_AOS, MF_HOST));
    xyz_host.resize(3 * _np, np ? xyz_host[3 * np - 1] : 0.f);
    check(mf_set_positions(handle_, xyz_host.data(), int64_t(_np), MF_LAYOUT_AOS, MF_HOST));
    refresh();
  }
  void setHext(const setHextParams& s) {
    check(mf_set_external(handle_, s.const_ext_field, reinterpret_cast<const float*>(s.ext_source_pos.data()),
                          reinterpret_cast<const float*>(s.ext_source_M.data()), int64_t(s.ext_source_pos.size()),
                          s.ext_mag_h));
  }
  void setTargetpos(const std::vector<float3>& pos) {
    check(mf_set_positions(handle_, reinterpret_cast<const float*>(pos.data()), int64_t(pos.size()),
                           MF_LAYOUT_AOS, MF_HOST));
    refresh();
  }
  void solve(size_t niter) {
    push_knobs();
    int64_t it = 0;
    double err = 0;
    mf_status st = mf_solve(handle_, int64_t(niter), &it, &err);
    if (st != MF_OK && st != MF_ERR_NOT_CONVERGED) check(st);
    i_step = size_t(it);
    int64_t len = 0;
    mf_get_error_history(handle_, nullptr, 0, &len);
    std::vector<double> hist(static_cast<size_t>(len));
    mf_get_error_history(handle_, hist.data(), len, &len);
    total_error.assign(hist.begin(), hist.end());
    refresh();
  }
  void evaluate_fitted_near_foece() {
    push_knobs();
    check(mf_eval_force(handle_));
    refresh();
  }
  void clear() {
    total_error.clear();
    i_step = 0;
  }
  void export_data(const char* path) { check(mf_export_data(handle_, path)); }
  void export_force(const char* path) { check(mf_export_force(handle_, path)); }

  mf_solver* handle() const { return handle_; }

  // Data (magnetic_force.cuh:116-173) -------------------------------------------
  float tolerance = 0.1f;     // magnetic_force.cu:626
  size_t max_iteration = 80;  // magnetic_force.cu:627
  size_t i_step = 0;
  std::vector<float> total_error;
  size_t np = 0;
  float chi = 0;
  float h = 0;
  float volume = 0;
  cuda_abstract_vector<float> xyz;
  cuda_abstract_vector<float> Hext;
  cuda_abstract_vector<float> M;
  cuda_abstract_vector<float> total_B_over_mu0;
  cuda_abstract_vector<float> dHextdx;
  cuda_abstract_vector<float> dHextdy;
  cuda_abstract_vector<float> dHextdz;
  cuda_abstract_vector<float> magnetic_bodyforce;
  bool naive = false;         // magnetic_force.cu:702
  int crit_size = 384;        // magnetic_force.cu:647

 private:
  static void check(mf_status s) {
    if (s != MF_OK) throw std::runtime_error(std::string(mf_status_string(s)) + ": " + mf_last_error());
  }
  void push_knobs() {
    check(mf_set_option(handle_, MF_OPT_TOLERANCE, double(tolerance)));
    check(mf_set_option(handle_, MF_OPT_MAX_ITERATION, double(max_iteration)));
    check(mf_set_option(handle_, MF_OPT_NAIVE, naive ? 1.0 : 0.0));
    check(mf_set_option(handle_, MF_OPT_CRIT_SIZE, double(crit_size)));
  }
  void view(int q, cuda_abstract_vector<float>& v) {
    check(mf_device_soa(handle_, q, &v.dev_x, &v.dev_y, &v.dev_z));
    v.np = np;
    v.owner = handle_;
    v.quantity = q;
  }
  void refresh() {
    int64_t n = 0;
    check(mf_num_particles(handle_, &n));
    np = size_t(n);
    view(MF_Q_POSITIONS, xyz);
    view(MF_Q_HEXT, Hext);
    view(MF_Q_M, M);
    view(MF_Q_B_OVER_MU0, total_B_over_mu0);
    view(MF_Q_DHEXTDX, dHextdx);
    view(MF_Q_DHEXTDY, dHextdy);
    view(MF_Q_DHEXTDZ, dHextdz);
    view(MF_Q_FORCE, magnetic_bodyforce);
  }
  mf_solver* handle_ = nullptr;
};

}  // namespace Libo
#endif  // LIBO_MAGNETIC_FORCE_SOLVER
