// mf_fmm.cu -- uniform-octree fast multipole method for the field and force
// products of large scenes.
//
// The reference evaluates large products with FMMTL (KernelMatrix.hpp:26-164,
// DualTraversal.hpp:80-125, BatchNear.hpp:57-75): an adaptive octree,
// spherical expansions in FP64 on the host CPU and a GPU near field.  Here the
// whole product stays on the device:
//   * one uniform box grid per level (level 0 is one box around the scene);
//     the leaf level is the deepest with >= leaf_min particles per box on
//     average, so a leaf box fills a 128-thread block of the near-field kernel;
//   * particles binned into leaf boxes in row-major order (x fastest), each
//     box's list in increasing particle index and padded to an even length,
//     so every run of x-adjacent boxes is one contiguous, pair-aligned range of
//     sources for the packed two-source pair body;
//   * Cartesian Taylor expansions of the dipole potential
//       phi(x) = 1/(4 pi) sum_j m_j . (x - y_j) / |x - y_j|^3
//     (multipoles and locals of degree 1..Q, Q = P - 1, M2L truncated at
//     |alpha| + |beta| <= Q + 1), each level's coefficients scaled by its box
//     edge so M2M, M2L and L2L do not depend on the level;
//   * box pairs accepted by the criterion of FMMOptions.hpp:56-78 (theta on
//     the box radii, with the separation test that the reference enables) are
//     far only if their gap also exceeds the kernel's near radius 4h, so every
//     far pair is in the pure-dipole regime of Dipole_B.kern:46-104 /
//     Dipole_hessian.kern:155-207 and the truncation is the only approximation;
//   * near leaf boxes (not accepted at the leaf level) are summed with the
//     packed clamped pair body of the all-pairs kernel, and the cell-list
//     correction (mf_cells.cu) turns the clamped pairs inside the near radius
//     into the reference's SPH / fitted-curve kernel.
// Every launch reads a solver stop flag and does nothing once it is set.
#include <algorithm>
#include <cmath>
#include <map>
#include <memory>
#include <new>
#include <tuple>
#include <type_traits>
#include <utility>
#include <vector>

#include "mf_internal.h"
#include "mf_sym.cuh"

namespace mfgb {
namespace {

constexpr int kMaxDegree = 9;  // P = 10 (the field products stop at degree 8)
constexpr int kMaxFieldDegree = 8;
constexpr int kMaxLevel = 10;

// Multi-indices in graded order: degree n, then s = y + z, then z.
__host__ __device__ constexpr int ncoef(int q) { return q < 0 ? 0 : (q + 1) * (q + 2) * (q + 3) / 6; }
__host__ __device__ constexpr int gidx(int x, int y, int z) {
  return ncoef(x + y + z - 1) + (y + z) * (y + z + 1) / 2 + z;
}

// Multi-index table up to degree kMaxDegree + 1.
__constant__ char4 c_mi[ncoef(kMaxDegree + 1)];
// 1-D translation factors: c_shift[c][j] = ((c - 1/2) / 2)^j / j!, the child
// centre offset in parent box units raised to j over j!.
__constant__ float c_shift[2][kMaxDegree + 2];

// ---------------------------------------------------------------------------
// Binning
// ---------------------------------------------------------------------------
__device__ __forceinline__ int64_t leaf_of(const FmmLevel& lv, float4 p) {
  const float inv = 1.f / lv.side;
  const int ix = min(max(int(floorf((p.x - lv.ox) * inv)), 0), lv.nx - 1);
  const int iy = min(max(int(floorf((p.y - lv.oy) * inv)), 0), lv.ny - 1);
  const int iz = min(max(int(floorf((p.z - lv.oz) * inv)), 0), lv.nz - 1);
  return (int64_t(iz) * lv.ny + iy) * lv.nx + ix;
}

__global__ void k_fmm_count(const float4* __restrict__ pos, int64_t n, FmmLevel lv, int32_t* __restrict__ cell_of,
                            int32_t* __restrict__ cnt) {
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
    const int64_t c = leaf_of(lv, pos[i]);
    cell_of[i] = int32_t(c);
    atomicAdd(&cnt[c], 1);
  }
}

// Exclusive scan of the even-padded counts into start[0..n], one CTA.
__global__ void __launch_bounds__(1024) k_fmm_scan(const int32_t* __restrict__ cnt, int64_t n,
                                                   int32_t* __restrict__ start) {
  __shared__ int32_t sh[1024];
  const int t = threadIdx.x;
  const int64_t chunk = (n + 1023) / 1024;
  const int64_t b = t * chunk, e = min(n, b + chunk);
  int32_t s = 0;
  for (int64_t i = b; i < e; ++i) s += cnt[i] + (cnt[i] & 1);
  sh[t] = s;
  __syncthreads();
  for (int o = 1; o < 1024; o <<= 1) {
    const int32_t v = t >= o ? sh[t - o] : 0;
    __syncthreads();
    sh[t] += v;
    __syncthreads();
  }
  int32_t run = sh[t] - s;
  for (int64_t i = b; i < e; ++i) {
    start[i] = run;
    run += cnt[i] + (cnt[i] & 1);
  }
  if (t == 1023) start[n] = sh[1023];
}

__global__ void k_fmm_scatter(const int32_t* __restrict__ cell_of, int64_t n, int32_t* __restrict__ cursor,
                              int32_t* __restrict__ tmp) {
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
    tmp[atomicAdd(&cursor[cell_of[i]], 1)] = int32_t(i);
}

// Each box's list in increasing particle index (one warp per box ranks its
// entries), then -1 in the padding slot of an odd box.
__global__ void k_fmm_sort(const int32_t* __restrict__ start, const int32_t* __restrict__ cnt, int64_t ncell,
                           const int32_t* __restrict__ tmp, int32_t* __restrict__ perm) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = int64_t(gridDim.x) * (blockDim.x >> 5);
  for (int64_t c = int64_t(blockIdx.x) * (blockDim.x >> 5) + (threadIdx.x >> 5); c < ncell; c += warps) {
    const int32_t b = start[c], m = cnt[c];
    for (int32_t k = lane; k < m; k += 32) {
      const int32_t v = tmp[b + k];
      int32_t rank = 0;
      for (int32_t l = 0; l < m; ++l) rank += tmp[b + l] < v;
      perm[b + rank] = v;
    }
    if (lane == 0 && (m & 1)) perm[b + m] = -1;
  }
}

// Occupancy of a level from its children's.
__global__ void k_fmm_occ_up(FmmLevel lc, FmmLevel lp, int32_t* __restrict__ occ) {
  for (int64_t b = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; b < lp.nbox; b += int64_t(gridDim.x) * blockDim.x) {
    const int px = int(b % lp.nx), py = int((b / lp.nx) % lp.ny), pz = int(b / (int64_t(lp.nx) * lp.ny));
    int32_t s = 0;
    for (int ch = 0; ch < 8; ++ch) {
      const int x = 2 * px + (ch & 1), y = 2 * py + ((ch >> 1) & 1), z = 2 * pz + (ch >> 2);
      if (x < lc.nx && y < lc.ny && z < lc.nz) s += occ[lc.box_off + (int64_t(z) * lc.ny + y) * lc.nx + x];
    }
    occ[lp.box_off + b] = s;
  }
}

// Sorted records in pair layout: slots 2p, 2p+1 as (x_a, x_b, y_a, y_b),
// (z_a, z_b, 0, 0).  A padding slot (always the odd one) repeats its
// partner's position (pos) or holds a zero dipole (moments).
__global__ void k_fmm_gather_pairs(const int32_t* __restrict__ perm, const float4* __restrict__ src,
                                   const int32_t* __restrict__ n_slots, float4* __restrict__ dst, int is_pos,
                                   const double* __restrict__ done) {
  if (done && *done != 0.0) return;
  const int64_t n_pairs = *n_slots / 2;
  for (int64_t p = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; p < n_pairs;
       p += int64_t(gridDim.x) * blockDim.x) {
    const int32_t ia = perm[2 * p], ib = perm[2 * p + 1];
    const float4 A = src[ia];
    const float4 B = ib >= 0 ? src[ib] : (is_pos ? A : make_float4(0.f, 0.f, 0.f, 0.f));
    dst[2 * p] = make_float4(A.x, B.x, A.y, B.y);
    dst[2 * p + 1] = make_float4(A.z, B.z, 0.f, 0.f);
  }
}

// Executed near-field pairs (real targets x real sources) and the largest leaf.
__global__ void k_fmm_p2p_stats(FmmLevel lv, const int32_t* __restrict__ cnt, const int32_t* __restrict__ tcnt,
                                const int4* __restrict__ rows, int n_rows, unsigned long long* __restrict__ out) {
  for (int64_t c = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; c < lv.nbox; c += int64_t(gridDim.x) * blockDim.x) {
    const int32_t n = tcnt[c];
    if (n == 0) continue;
    const int ix = int(c % lv.nx), iy = int((c / lv.nx) % lv.ny), iz = int(c / (int64_t(lv.nx) * lv.ny));
    unsigned long long s = 0;
    for (int r = 0; r < n_rows; ++r) {
      const int4 rw = rows[r];
      const int cy = iy + rw.y, cz = iz + rw.z;
      if (cy < 0 || cy >= lv.ny || cz < 0 || cz >= lv.nz) continue;
      const int cx0 = max(ix - rw.x, 0), cx1 = min(ix + rw.x, lv.nx - 1);
      const int64_t rb = (int64_t(cz) * lv.ny + cy) * lv.nx;
      for (int x = cx0; x <= cx1; ++x) s += unsigned(cnt[rb + x]);
    }
    atomicAdd(&out[0], s * unsigned(n));
    atomicMax(&out[1], (unsigned long long)n);
    atomicAdd(&out[3], 1ull);
    atomicAdd(&out[4], (unsigned long long)cnt[c] * unsigned(n));
  }
}

// Multipole-to-local translations of one level (target box holding targets,
// source box holding sources), one warp per target box.
__global__ void k_fmm_m2l_stats(FmmLevel lv, const int32_t* __restrict__ occ, const int32_t* __restrict__ tocc,
                                const int4* __restrict__ list, const int64_t* __restrict__ off,
                                const int64_t* __restrict__ cnt, unsigned long long* __restrict__ out) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = int64_t(gridDim.x) * (blockDim.x >> 5);
  for (int64_t b = int64_t(blockIdx.x) * (blockDim.x >> 5) + (threadIdx.x >> 5); b < lv.nbox; b += warps) {
    if (tocc[lv.box_off + b] == 0) continue;
    const int x = int(b % lv.nx), y = int((b / lv.nx) % lv.ny), z = int(b / (int64_t(lv.nx) * lv.ny));
    const int cls = (x & 1) | ((y & 1) << 1) | ((z & 1) << 2);
    unsigned k = 0;
    for (int64_t e = off[cls] + lane; e < off[cls] + cnt[cls]; e += 32) {
      const int4 d = list[e];
      const int sx = x - d.x, sy = y - d.y, sz = z - d.z;
      if (unsigned(sx) >= unsigned(lv.nx) || unsigned(sy) >= unsigned(lv.ny) || unsigned(sz) >= unsigned(lv.nz)) continue;
      k += occ[lv.box_off + (int64_t(sz) * lv.ny + sy) * lv.nx + sx] > 0 ? 1u : 0u;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) k += __shfl_xor_sync(0xffffffffu, k, o);
    if (lane == 0) atomicAdd(&out[2], (unsigned long long)k);
  }
}

// ---------------------------------------------------------------------------
// Upward pass
// ---------------------------------------------------------------------------
// Leaf multipoles, one CTA per box, one thread per coefficient alpha (two for
// degree 8, whose 164 coefficients outnumber the threads):
//   M_alpha = (-1)^|alpha| sum_j sum_k m_jk u_j^(alpha - e_k) / (alpha - e_k)!,
// u_j = (y_j - centre) / edge.
template <int Q>
__global__ void __launch_bounds__(128) k_fmm_p2m(FmmLevel lv, const int32_t* __restrict__ start,
                                                 const int32_t* __restrict__ cnt, const int32_t* __restrict__ perm,
                                                 const float4* __restrict__ pos4, const float4* __restrict__ mom4,
                                                 float* __restrict__ M, const double* __restrict__ done) {
  constexpr int NC = ncoef(Q) - 1;
  constexpr int KPT = (NC + 127) / 128;  // coefficients per thread
  constexpr int W = 3 * Q + 3;  // powers u^i/i! (i < Q) per axis, then the dipole
  if (done && *done != 0.0) return;
  __shared__ float s_p[128][W + 1];
  const int tid = threadIdx.x;
  bool act[KPT];
  int ax[KPT], ay[KPT], az[KPT];
  float sign[KPT];
#pragma unroll
  for (int r = 0; r < KPT; ++r) {
    const int k = tid + 128 * r;
    act[r] = k < NC;
    ax[r] = ay[r] = az[r] = 0;
    if (act[r]) {
      const char4 e = c_mi[k + 1];
      ax[r] = e.x;
      ay[r] = e.y;
      az[r] = e.z;
    }
    sign[r] = ((ax[r] + ay[r] + az[r]) & 1) ? -1.f : 1.f;
  }
  const float inv_s = 1.f / lv.side;
  for (int64_t c = blockIdx.x; c < lv.nbox; c += gridDim.x) {
    const int32_t n = cnt[c];
    float acc[KPT];
#pragma unroll
    for (int r = 0; r < KPT; ++r) acc[r] = 0.f;
    if (n > 0) {
      const int ix = int(c % lv.nx), iy = int((c / lv.nx) % lv.ny), iz = int(c / (int64_t(lv.nx) * lv.ny));
      const float cx = lv.ox + (float(ix) + 0.5f) * lv.side;
      const float cy = lv.oy + (float(iy) + 0.5f) * lv.side;
      const float cz = lv.oz + (float(iz) + 0.5f) * lv.side;
      const int32_t b = start[c];
      for (int j0 = 0; j0 < n; j0 += 128) {
        const int nj = min(128, n - j0);
        __syncthreads();
        if (tid < nj) {
          const int32_t i = perm[b + j0 + tid];
          const float4 p = pos4[i], m = mom4[i];
          const float u[3] = {(p.x - cx) * inv_s, (p.y - cy) * inv_s, (p.z - cz) * inv_s};
#pragma unroll
          for (int a = 0; a < 3; ++a) {
            float v = 1.f;
            s_p[tid][a * Q] = 1.f;
#pragma unroll
            for (int k = 1; k < Q; ++k) {
              v = v * u[a] * (1.f / float(k));
              s_p[tid][a * Q + k] = v;
            }
          }
          s_p[tid][3 * Q] = m.x;
          s_p[tid][3 * Q + 1] = m.y;
          s_p[tid][3 * Q + 2] = m.z;
        }
        __syncthreads();
#pragma unroll
        for (int r = 0; r < KPT; ++r) {
          if (act[r]) {
            for (int j = 0; j < nj; ++j) {
              const float* q = s_p[j];
              float t = 0.f;
              if (ax[r] > 0) t += q[3 * Q] * q[ax[r] - 1] * q[Q + ay[r]] * q[2 * Q + az[r]];
              if (ay[r] > 0) t += q[3 * Q + 1] * q[ax[r]] * q[Q + ay[r] - 1] * q[2 * Q + az[r]];
              if (az[r] > 0) t += q[3 * Q + 2] * q[ax[r]] * q[Q + ay[r]] * q[2 * Q + az[r] - 1];
              acc[r] += t;
            }
          }
        }
      }
    }
#pragma unroll
    for (int r = 0; r < KPT; ++r)
      if (act[r]) M[int64_t(tid + 128 * r) * lv.nbox + c] = sign[r] * acc[r];
  }
}

// Children -> parent:  M^p_alpha = sum_c sum_{gamma <= alpha}
//   2^(1-|gamma|) M^c_gamma (-1)^|delta| v_c^delta / delta!,  delta = alpha - gamma,
// v_c the child centre offset in parent box units.  One thread per (alpha, box).
template <int Q>
__global__ void k_fmm_m2m(FmmLevel lc, FmmLevel lp, const int32_t* __restrict__ occ, float* __restrict__ M,
                          const double* __restrict__ done) {
  constexpr int NC = ncoef(Q) - 1;
  if (done && *done != 0.0) return;
  const float* Mc = M + lc.box_off * NC;
  float* Mp = M + lp.box_off * NC;
  for (int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; t < int64_t(NC) * lp.nbox;
       t += int64_t(gridDim.x) * blockDim.x) {
    const int k = int(t / lp.nbox);
    const int64_t b = t % lp.nbox;
    float acc = 0.f;
    if (occ[lp.box_off + b] > 0) {
      const char4 e = c_mi[k + 1];
      const int px = int(b % lp.nx), py = int((b / lp.nx) % lp.ny), pz = int(b / (int64_t(lp.nx) * lp.ny));
      for (int ch = 0; ch < 8; ++ch) {
        const int cx = ch & 1, cy = (ch >> 1) & 1, cz = ch >> 2;
        const int x = 2 * px + cx, y = 2 * py + cy, z = 2 * pz + cz;
        if (x >= lc.nx || y >= lc.ny || z >= lc.nz) continue;
        const int64_t cb = (int64_t(z) * lc.ny + y) * lc.nx + x;
        if (occ[lc.box_off + cb] == 0) continue;
        for (int gx = 0; gx <= e.x; ++gx)
          for (int gy = 0; gy <= e.y; ++gy)
            for (int gz = 0; gz <= e.z; ++gz) {
              const int g = gx + gy + gz;
              if (g == 0) continue;
              const int dx = e.x - gx, dy = e.y - gy, dz = e.z - gz;
              // (-1)^|delta| v^delta / delta! = prod over axes of ((1/2 - c) / 2)^d / d!
              const float w = c_shift[1 - cx][dx] * c_shift[1 - cy][dy] * c_shift[1 - cz][dz];
              acc += Mc[int64_t(gidx(gx, gy, gz) - 1) * lc.nbox + cb] * w * ldexpf(1.f, 1 - g);
            }
      }
    }
    Mp[int64_t(k) * lp.nbox + b] = acc;
  }
}

// ---------------------------------------------------------------------------
// M2L:  L_beta += sum_alpha M_alpha D_(alpha + beta)(d),  |alpha| + |beta| <= Q + 1,
// D_gamma(d) = d^gamma (1/|d|) at the box-centre offset d in box units.  The
// sum is an unrolled program over compile-time (gamma, alpha, beta) triples,
// gamma-major so each D value is loaded once; beta degrees BLO..BHI per
// variant (two variants split the largest degrees so the multipole and the
// accumulators both stay in registers).
// ---------------------------------------------------------------------------
template <int Q, int BLO, int BHI>
struct M2LPlan {
  static constexpr int AMAX = (Q < Q + 1 - BLO) ? Q : Q + 1 - BLO;
  static constexpr int NA = ncoef(AMAX) - 1;
  static constexpr int BOFF = ncoef(BLO - 1);
  static constexpr int NB = ncoef(BHI) - ncoef(BLO - 1);
  struct Ent {
    int16_t g, a, b, first;
  };
  static constexpr int count() {
    int k = 0;
    for (int g = BLO + 1; g <= Q + 1; ++g)
      for (int s = 0; s <= g; ++s)
        for (int gz = 0; gz <= s; ++gz) {
          const int gy = s - gz, gx = g - s;
          for (int ax = 0; ax <= gx; ++ax)
            for (int ay = 0; ay <= gy; ++ay)
              for (int az = 0; az <= gz; ++az) {
                const int a = ax + ay + az, b = g - a;
                if (a >= 1 && a <= AMAX && b >= BLO && b <= BHI) ++k;
              }
        }
    return k;
  }
  static constexpr int K = count();
  struct Tab {
    Ent e[K];
  };
  static constexpr Tab make() {
    Tab t{};
    int k = 0;
    for (int g = BLO + 1; g <= Q + 1; ++g)
      for (int s = 0; s <= g; ++s)
        for (int gz = 0; gz <= s; ++gz) {
          const int gy = s - gz, gx = g - s;
          bool first = true;
          for (int ax = 0; ax <= gx; ++ax)
            for (int ay = 0; ay <= gy; ++ay)
              for (int az = 0; az <= gz; ++az) {
                const int a = ax + ay + az, b = g - a;
                if (a >= 1 && a <= AMAX && b >= BLO && b <= BHI) {
                  t.e[k].g = int16_t(gidx(gx, gy, gz));
                  t.e[k].a = int16_t(gidx(ax, ay, az) - 1);
                  t.e[k].b = int16_t(gidx(gx - ax, gy - ay, gz - az) - BOFF);
                  t.e[k].first = int16_t(first ? 1 : 0);
                  first = false;
                  ++k;
                }
              }
        }
    return t;
  }
  static constexpr Tab tab = make();
  template <int I>
  struct At {
    static constexpr int g = tab.e[I].g, a = tab.e[I].a, b = tab.e[I].b, first = tab.e[I].first;
  };
};

template <class Pl, int I>
__device__ __forceinline__ void m2l_step(float* acc, const float* M, const float* __restrict__ dt, float& dg) {
  using E = typename Pl::template At<I>;
  if constexpr (E::first != 0) dg = __ldg(dt + E::g);
  acc[E::b] = fmaf(M[E::a], dg, acc[E::b]);
}

template <class Pl, int... Is>
__device__ __forceinline__ void m2l_apply(float* acc, const float* M, const float* __restrict__ dt,
                                          std::integer_sequence<int, Is...>) {
  float dg = 0.f;
  (m2l_step<Pl, Is>(acc, M, dt, dg), ...);
}

struct M2LArgs {
  FmmLevel lv;
  const int32_t* occ;   // sources per box
  const int32_t* tocc;  // targets per box
  const float* M;     // this level's multipoles (NC rows of nbox)
  float* Lp;          // [chunks][NC][nbox] partial locals
  const int4* list;   // (dx, dy, dz, row of dtab)
  const float* dtab;  // [rows][ncoef(Q + 1)]
  int64_t list_off[8];
  int32_t list_cnt[8];
  int32_t chunks;
  int32_t hx, hy, hz;  // half-grid extents (boxes per class along each axis)
  int64_t per_class;   // hx * hy * hz rounded up to a multiple of 32
  const double* done;
};

// One thread per (list chunk, target box); the warps of a block share the
// chunk and the target parity class, so they walk the same offsets.
template <int Q, int BLO, int BHI>
__global__ void __launch_bounds__(128) k_fmm_m2l(const M2LArgs p) {
  using Pl = M2LPlan<Q, BLO, BHI>;
  constexpr int NC = ncoef(Q) - 1;
  constexpr int NG = ncoef(Q + 1);
  if (p.done && *p.done != 0.0) return;
  const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const int64_t per = p.per_class;
  const int ch = int(t / (8 * per));
  if (ch >= p.chunks) return;
  const int cls = int((t / per) % 8);
  const int64_t r = t % per;
  const int hi = int(r % p.hx), hj = int((r / p.hx) % p.hy);
  const int64_t hk = r / (int64_t(p.hx) * p.hy);
  if (hk >= p.hz) return;
  const FmmLevel& lv = p.lv;
  const int tx = 2 * hi + (cls & 1), ty = 2 * hj + ((cls >> 1) & 1), tz = 2 * int(hk) + (cls >> 2);
  if (tx >= lv.nx || ty >= lv.ny || tz >= lv.nz) return;
  const int64_t tb = (int64_t(tz) * lv.ny + ty) * lv.nx + tx;
  if (p.tocc[lv.box_off + tb] == 0) return;
  const int64_t n = p.list_cnt[cls];
  const int64_t e0 = p.list_off[cls] + n * ch / p.chunks;
  const int64_t e1 = p.list_off[cls] + n * (ch + 1) / p.chunks;
  float acc[Pl::NB];
#pragma unroll
  for (int q = 0; q < Pl::NB; ++q) acc[q] = 0.f;
  for (int64_t e = e0; e < e1; ++e) {
    const int4 d = __ldg(p.list + e);
    const int sx = tx - d.x, sy = ty - d.y, sz = tz - d.z;
    if (unsigned(sx) >= unsigned(lv.nx) || unsigned(sy) >= unsigned(lv.ny) || unsigned(sz) >= unsigned(lv.nz))
      continue;
    const int64_t sb = (int64_t(sz) * lv.ny + sy) * lv.nx + sx;
    if (__ldg(p.occ + lv.box_off + sb) == 0) continue;
    float M[Pl::NA];
#pragma unroll
    for (int q = 0; q < Pl::NA; ++q) M[q] = __ldg(p.M + int64_t(q) * lv.nbox + sb);
    m2l_apply<Pl>(acc, M, p.dtab + int64_t(d.w) * NG, std::make_integer_sequence<int, Pl::K>{});
  }
  float* out = p.Lp + int64_t(ch) * NC * lv.nbox;
#pragma unroll
  for (int q = 0; q < Pl::NB; ++q) out[int64_t(Pl::BOFF - 1 + q) * lv.nbox + tb] = acc[q];
}

// Locals of a level: the M2L partials plus the parent's locals shifted to the
// child centre,  L^c_beta += 2^(-2-|beta|) sum_delta L^p_(beta+delta) v_c^delta / delta!.
// `occ` counts targets: boxes without targets need no locals.
// kmin: coefficients below it are not computed (zero): a Hessian-only product
// has no degree-1 partials (kmin 3).
template <int Q>
__global__ void k_fmm_l2l(FmmLevel lv, FmmLevel lp, int has_parent, const int32_t* __restrict__ occ,
                          const float* __restrict__ Lpart, int chunks, float* __restrict__ L,
                          const double* __restrict__ done, int kmin) {
  constexpr int NC = ncoef(Q) - 1;
  if (done && *done != 0.0) return;
  const float* Lpar = L + lp.box_off * NC;
  float* Lout = L + lv.box_off * NC;
  for (int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; t < int64_t(NC) * lv.nbox;
       t += int64_t(gridDim.x) * blockDim.x) {
    const int k = int(t / lv.nbox);
    const int64_t b = t % lv.nbox;
    float v = 0.f;
    if (k >= kmin && occ[lv.box_off + b] > 0) {
      for (int ch = 0; ch < chunks; ++ch) v += Lpart[(int64_t(ch) * NC + k) * lv.nbox + b];
      if (has_parent) {
        const char4 e = c_mi[k + 1];
        const int deg = e.x + e.y + e.z;
        const int x = int(b % lv.nx), y = int((b / lv.nx) % lv.ny), z = int(b / (int64_t(lv.nx) * lv.ny));
        const int64_t pb = (int64_t(z >> 1) * lp.ny + (y >> 1)) * lp.nx + (x >> 1);
        const int cx = x & 1, cy = y & 1, cz = z & 1;
        float s = 0.f;
        for (int dx = 0; dx <= Q - deg; ++dx)
          for (int dy = 0; dy <= Q - deg - dx; ++dy)
            for (int dz = 0; dz <= Q - deg - dx - dy; ++dz)
              s += Lpar[int64_t(gidx(e.x + dx, e.y + dy, e.z + dz) - 1) * lp.nbox + pb] * c_shift[cx][dx] *
                   c_shift[cy][dy] * c_shift[cz][dz];
        v += ldexpf(s, -2 - deg);
      }
    }
    Lout[int64_t(k) * lv.nbox + b] = v;
  }
}

// ---------------------------------------------------------------------------
// Near field + L2P + epilogue: one CTA per leaf box, one target per thread.
// Source runs (rows of x-adjacent near boxes) are cut into tiles staged in
// shared memory by bulk copies on an mbarrier pipeline, as in the all-pairs
// kernel, and swept with the packed clamped pair body.
// ---------------------------------------------------------------------------
// The CTA shape (threads per leaf box, one target each with rounds for
// larger boxes; sources per stage) is a template parameter of the kernel.
constexpr int kP2PStages = 3;
constexpr int kP2PMaxSteps = 128;  // tile steps per refill of the row walk (1 KB of shared memory)
template <int TILE>
constexpr int p2p_smem() { return kP2PStages * 2 * TILE * int(sizeof(float4)); }

struct P2PArgs {
  FmmLevel lv;
  const int32_t* start;   // sources: box starts (even-padded slots), counts, slot -> index
  const int32_t* cnt;
  const int32_t* perm;
  const int32_t* tstart;  // targets: box starts, counts, slot -> index (the same arrays
  const int32_t* tcnt;    //   when the targets are the sources)
  const int32_t* tperm;
  const float4* pos2s;
  const float4* mom2s;
  const float* L;     // leaf locals, NC rows of nbox
  const int4* rows;   // (half-width w, dy, dz, 0)
  int32_t n_rows;
  const double* done;
  // Near field from partial sums (k_fmm_near_sym): the half-stencil rows,
  // the planes [1 + offsets][3][n_slots] and their slot count.
  const int4* hrows;
  int32_t n_hrows;
  const float* part;
  int64_t n_slots;
};

// Plane of box offset dx in half row hr (1 + offsets before the row + index).
__device__ __forceinline__ int near_plane(const int4& hr, int dx) {
  return 1 + hr.w + ((hr.y == 0 && hr.z == 0) ? dx - 1 : dx + hr.x);
}

// kKind: 0 field (H), 1 Kelvin force (contracted with the target dipole),
// 2 force tensor (the Hessian kernel's 3x3 at each target).
// kParts (force, targets = sources): the near field is not swept here but
// added from k_fmm_near_sym's partial sums -- the box's own plane, then the
// plane of every writer box (this box minus a half-stencil offset, inside the
// grid and not empty), in a fixed order with compensated FP32.
template <int Q, int kKind, bool kParts, int TPB, int TILE>
__global__ void __launch_bounds__(TPB) k_fmm_p2p(const P2PArgs p, const AllPairsArgs<float> a,
                                                         const SceneDesc<float> sc) {
  static_assert(!kParts || kKind == 1, "partial sums: the Kelvin force only");
  using Body = std::conditional_t<kKind == 0, FieldF2Body, std::conditional_t<kKind == 1, ForceF2Body, TensorF2Body>>;
  constexpr bool kForce = kKind == 1;
  constexpr int kOut = Body::kOut;
  constexpr int NC = ncoef(Q) - 1;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t bar[kP2PStages];
  __shared__ int2 s_steps[kP2PMaxSteps];
  __shared__ int s_nsteps, s_row, s_pos;
  __shared__ float s_L[NC];
  if (p.done && *p.done != 0.0) return;
  const FmmLevel& lv = p.lv;
  const int64_t c = blockIdx.x;
  const int32_t n = p.tcnt[c];
  if (n == 0) return;
  const int tid = threadIdx.x;
  const int ix = int(c % lv.nx), iy = int((c / lv.nx) % lv.ny), iz = int(c / (int64_t(lv.nx) * lv.ny));
  const int32_t st0 = p.tstart[c];
  for (int k = tid; k < NC; k += TPB) s_L[k] = p.L[int64_t(k) * lv.nbox + c];
  auto stage_pos = [&](int s) { return reinterpret_cast<float4*>(smem_raw) + s * 2 * TILE; };
  auto stage_mom = [&](int s) { return stage_pos(s) + TILE; };
  if (tid == 0) {
    for (int s = 0; s < kP2PStages; ++s) mbar_init(&bar[s], 1);
    fence_mbar_init();
  }
  __syncthreads();

  auto issue = [&](int k, int s) {
    const int2 stp = s_steps[k];
    const uint32_t bytes = uint32_t(stp.y) * uint32_t(sizeof(float4));
    mbar_arrive_expect_tx(&bar[s], 2 * bytes);
    bulk_g2s(stage_pos(s), p.pos2s + stp.x, bytes, &bar[s]);
    bulk_g2s(stage_mom(s), p.mom2s + stp.x, bytes, &bar[s]);
  };
  // Thread 0: next tiles of the row walk into s_steps.
  auto fill = [&]() {
    int k = 0, r = s_row;
    int32_t pos = s_pos;
    while (r < p.n_rows && k < kP2PMaxSteps) {
      const int4 rw = p.rows[r];
      const int cy = iy + rw.y, cz = iz + rw.z;
      if (cy < 0 || cy >= lv.ny || cz < 0 || cz >= lv.nz) {
        ++r;
        pos = -1;
        continue;
      }
      const int cx0 = max(ix - rw.x, 0), cx1 = min(ix + rw.x, lv.nx - 1);
      const int64_t rb = (int64_t(cz) * lv.ny + cy) * lv.nx;
      const int32_t b = p.start[rb + cx0], e = p.start[rb + cx1 + 1];
      if (pos < 0) pos = b;
      if (pos >= e) {
        ++r;
        pos = -1;
        continue;
      }
      const int32_t m = min(TILE, e - pos);
      s_steps[k++] = make_int2(pos, m);
      pos += m;
    }
    s_row = r;
    s_pos = pos;
    s_nsteps = k;
  };

  uint32_t u = 0;  // steps consumed so far (stage and parity of the next)
  bool failed = false;
  int fail_k = 0, fail_ns = 0;
  for (int t0 = 0; t0 < n && !failed; t0 += TPB) {
    const bool act = t0 + tid < n;
    // A warp without a live target (the last warps of a small box) skips
    // the pair sweeps; it still takes part in every barrier and wait.
    const bool warp_live = __any_sync(0xffffffffu, act);
    const int32_t i = p.tperm[st0 + (act ? t0 + tid : 0)];
    typename Body::TData td;
    Body::load(a, i, td);
    float run[kOut], cmp[kOut];
#pragma unroll
    for (int q = 0; q < kOut; ++q) run[q] = cmp[q] = 0.f;
    if constexpr (kParts) {
      if (act) {
        const int64_t slot = int64_t(st0) + t0 + tid;
#pragma unroll
        for (int q = 0; q < 3; ++q) two_sum_acc(run[q], cmp[q], __ldcg(p.part + int64_t(q) * p.n_slots + slot));
        for (int r = 0; r < p.n_hrows; ++r) {
          const int4 hr = p.hrows[r];
          const int ay = iy - hr.y, az = iz - hr.z;
          if (ay < 0 || ay >= lv.ny || az < 0 || az >= lv.nz) continue;
          for (int dx = (hr.y == 0 && hr.z == 0) ? 1 : -hr.x; dx <= hr.x; ++dx) {
            const int ax = ix - dx;
            if (ax < 0 || ax >= lv.nx) continue;
            if (p.cnt[(int64_t(az) * lv.ny + ay) * lv.nx + ax] == 0) continue;
            const float* pl = p.part + int64_t(near_plane(hr, dx)) * 3 * p.n_slots + slot;
#pragma unroll
            for (int q = 0; q < 3; ++q) two_sum_acc(run[q], cmp[q], __ldcg(pl + int64_t(q) * p.n_slots));
          }
        }
      }
    }
    if (tid == 0) {
      s_row = 0;
      s_pos = -1;
    }
    // The row walk and its sweeps (not in the read-back mode).
    if constexpr (!kParts) for (;;) {
      __syncthreads();  // the previous segment's steps are consumed
      if (tid == 0) fill();
      __syncthreads();
      const int ns = s_nsteps;
      if (ns == 0) break;
      if (tid == 0)
        for (int k = 0; k < kP2PStages && k < ns; ++k) issue(k, int((u + k) % kP2PStages));
      for (int k = 0; k < ns; ++k) {
        const uint32_t uu = u + uint32_t(k);
        const int s = int(uu % kP2PStages);
        const bool ok = mbar_wait_bounded(&bar[s], (uu / kP2PStages) & 1u);
        if (__syncthreads_or(!ok)) {
          failed = true;
          fail_k = k;
          fail_ns = ns;
          break;
        }
        const int n_items = s_steps[k].y >> 1;
        const float4* __restrict__ sp = stage_pos(s);
        const float4* __restrict__ sm = stage_mom(s);
        if (warp_live) {
          typename Body::Acc acc;
          acc.zero();
#pragma unroll 4
          for (int j = 0; j < n_items; ++j) Body::pair(td, Body::load_item(sp, sm, j), sc.pc, acc);
          float o[kOut];
          Body::tile_out(acc, o);
#pragma unroll
          for (int q = 0; q < kOut; ++q) comp_add(run[q], cmp[q], o[q]);
        }
        __syncthreads();  // stage s is free
        if (tid == 0 && k + kP2PStages < ns) {
          fence_proxy_async_smem();
          issue(k + kP2PStages, s);
        }
      }
      if (failed) break;
      u += uint32_t(ns);
    }
    if (failed) break;
    __syncthreads();  // stages idle: reuse them for the power tables
    // Far field from the box's local expansion at w = (x - centre) / edge.
    float* pw = reinterpret_cast<float*>(smem_raw);  // [3Q][threads]
    const float4 tp = a.tpos[i];
    const float inv_s = 1.f / lv.side;
    const float w[3] = {(tp.x - (lv.ox + (float(ix) + 0.5f) * lv.side)) * inv_s,
                        (tp.y - (lv.oy + (float(iy) + 0.5f) * lv.side)) * inv_s,
                        (tp.z - (lv.oz + (float(iz) + 0.5f) * lv.side)) * inv_s};
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) {
      float v = 1.f;
      pw[(ax * Q) * TPB + tid] = 1.f;
#pragma unroll
      for (int k = 1; k < Q; ++k) {
        v = v * w[ax] * (1.f / float(k));
        pw[(ax * Q + k) * TPB + tid] = v;
      }
    }
    double v[kOut];
    for (int q = 0; q < kOut; ++q) v[q] = double(run[q]) + double(cmp[q]);
    if constexpr (kKind == 0) {
      // H = -grad phi = -1/(4 pi s^3) sum_g L_(g + e_k) w^g / g!
      float h0 = 0.f, h1 = 0.f, h2 = 0.f;
      for (int g = 0; g < ncoef(Q - 1); ++g) {
        const char4 e = c_mi[g];
        const float mono = pw[e.x * TPB + tid] * pw[(Q + e.y) * TPB + tid] *
                           pw[(2 * Q + e.z) * TPB + tid];
        h0 = fmaf(s_L[gidx(e.x + 1, e.y, e.z) - 1], mono, h0);
        h1 = fmaf(s_L[gidx(e.x, e.y + 1, e.z) - 1], mono, h1);
        h2 = fmaf(s_L[gidx(e.x, e.y, e.z + 1) - 1], mono, h2);
      }
      const double f = -kInv4Pi * double(inv_s) * double(inv_s) * double(inv_s);
      v[0] += f * double(h0);
      v[1] += f * double(h1);
      v[2] += f * double(h2);
    } else {
      // Hess phi = 1/(4 pi s^4) sum_g L_(g + e_a + e_b) w^g / g!;  F = -mu0 Hess phi m_t
      float hxx = 0.f, hyy = 0.f, hzz = 0.f, hxy = 0.f, hxz = 0.f, hyz = 0.f;
      for (int g = 0; g < ncoef(Q - 2); ++g) {
        const char4 e = c_mi[g];
        const float mono = pw[e.x * TPB + tid] * pw[(Q + e.y) * TPB + tid] *
                           pw[(2 * Q + e.z) * TPB + tid];
        hxx = fmaf(s_L[gidx(e.x + 2, e.y, e.z) - 1], mono, hxx);
        hyy = fmaf(s_L[gidx(e.x, e.y + 2, e.z) - 1], mono, hyy);
        hzz = fmaf(s_L[gidx(e.x, e.y, e.z + 2) - 1], mono, hzz);
        hxy = fmaf(s_L[gidx(e.x + 1, e.y + 1, e.z) - 1], mono, hxy);
        hxz = fmaf(s_L[gidx(e.x + 1, e.y, e.z + 1) - 1], mono, hxz);
        hyz = fmaf(s_L[gidx(e.x, e.y + 1, e.z + 1) - 1], mono, hyz);
      }
      const double is2 = double(inv_s) * double(inv_s);
      const double f = -kMu0 * kInv4Pi * is2 * is2;
      if constexpr (kForce) {
        const float4 tm = a.tmom[i];
        v[0] += f * (double(hxx) * tm.x + double(hxy) * tm.y + double(hxz) * tm.z);
        v[1] += f * (double(hxy) * tm.x + double(hyy) * tm.y + double(hyz) * tm.z);
        v[2] += f * (double(hxz) * tm.x + double(hyz) * tm.y + double(hzz) * tm.z);
      } else {
        // T = -mu0 Hess phi, entries xx, yy, zz, xy, xz, yz
        v[0] += f * double(hxx);
        v[1] += f * double(hyy);
        v[2] += f * double(hzz);
        v[3] += f * double(hxy);
        v[4] += f * double(hxz);
        v[5] += f * double(hyz);
      }
    }
    if (act) Body::epilogue(a, sc, i, td, v);
  }
  if (failed && tid == 0) {
    // Copies in flight: steps fail_k .. min(fail_ns, fail_k + stages) - 1 of
    // the segment that failed, one per stage; wait for each (bounded).
    atomicExch(a.err, MF_DEVERR_STAGE_TIMEOUT);
    bool drained = true;
    const int k_stop = min(fail_ns, fail_k + kP2PStages);
    for (int k = fail_k; k < k_stop; ++k) {
      const uint32_t uu = u + uint32_t(k);
      if (!mbar_wait_bounded(&bar[uu % kP2PStages], (uu / kP2PStages) & 1u)) drained = false;
    }
    if (!drained) atomicExch(a.err, MF_DEVERR_DRAIN_TIMEOUT);
  }
}

// ---------------------------------------------------------------------------
// Near field of the Kelvin force once per unordered box pair (targets are the
// sources): one warp per leaf box A.  Both half-warps hold the same 128
// target slots (8 per lane; rounds of 128 for larger boxes) and sweep
// alternate pairs of source items, so every shuffle tree of the source sums
// spans 16 lanes and serves 8 targets per lane.
//   * A's own pairs: every ordered pair, target side only.
//   * The boxes B of the half stencil: each pair item's force adds into the
//     targets' sums and, reduced over the half-warp by a fixed shuffle tree,
//     into the sources' sums (f_ji = -f_ij), stored at plane near_plane(B - A)
//     of the source's slot.  A later target round adds to the entries of the
//     earlier ones (the same lane, in order).
//   * The targets' sums (the two halves' added) go to plane 0.
// Every (plane, slot) entry has one writer, so results do not depend on
// scheduling.  Sums are in the all-pairs kernels' units (times K).
// ---------------------------------------------------------------------------
struct NearSymArgs {
  FmmLevel lv;
  const int32_t* start;  // box slot starts (even-padded), leaf level
  const int32_t* cnt;
  const int32_t* perm;   // slot -> particle
  const float4* pos2s;   // pair-layout records by slot
  const float4* mom2s;
  const int4* hrows;
  int32_t n_hrows;
  float* part;
  int64_t n_slots;
  const double* done;
};
constexpr int kNearSymWarps = 4, kNearSymTPT = 8, kNearSymChunk = 64;

// The walk over the half stencil's source boxes in units of up to
// kNearSymChunk pair items (a box in one or more chunks), in the order
// rows, x offsets, chunks.
struct NearUnit {
  int32_t sb;     // first slot of the box
  int32_t cs;     // first item of the chunk in the box
  int32_t cn;     // items in the chunk
  int32_t plane;  // partial-sum plane of the box's offset (-1: no unit)
};
struct NearCursor {
  int r, dx;         // next half-stencil row and x offset to examine
  int32_t sb, ni;    // the box being chunked (ni items; 0: none)
  int32_t cs, plane;
};

__device__ __forceinline__ NearUnit near_next(NearCursor& cur, const NearSymArgs& p, int ix, int iy, int iz) {
  constexpr int CH = kNearSymChunk;
  const FmmLevel& lv = p.lv;
  for (;;) {
    if (cur.cs < cur.ni) {
      const NearUnit u{cur.sb, cur.cs, min(CH, cur.ni - cur.cs), cur.plane};
      cur.cs += CH;
      return u;
    }
    if (cur.r >= p.n_hrows) return NearUnit{0, 0, 0, -1};
    const int4 hr = p.hrows[cur.r];
    const int cy = iy + hr.y, cz = iz + hr.z;
    const int dx = cur.dx;
    if (cy < 0 || cy >= lv.ny || cz < 0 || cz >= lv.nz || dx > hr.x) {  // next row
      ++cur.r;
      if (cur.r < p.n_hrows) {
        const int4 h2 = p.hrows[cur.r];
        cur.dx = (h2.y == 0 && h2.z == 0) ? 1 : -h2.x;
      }
      continue;
    }
    ++cur.dx;
    const int cx = ix + dx;
    if (cx < 0 || cx >= lv.nx) continue;
    const int64_t b = (int64_t(cz) * lv.ny + cy) * lv.nx + cx;
    const int32_t nb = p.cnt[b];
    if (nb == 0) continue;
    cur.sb = p.start[b];
    cur.ni = (nb + 1) >> 1;
    cur.cs = 0;
    cur.plane = near_plane(hr, dx);
  }
}

// Reduce-scatter of NV values over each half-warp (16 lanes): lane l ends
// with value l & 15 summed over its half, by a fixed shuffle tree.
template <int NV>
__device__ __forceinline__ float half_reduce_scatter(const float (&v)[NV], int lane) {
  static_assert(NV == 16, "one value per lane of a half-warp");
  float w[NV];
#pragma unroll
  for (int q = 0; q < NV; ++q) w[q] = v[q];
  int b = 8;
#pragma unroll
  for (int n = NV; n > 1; n >>= 1, b >>= 1) {
    const bool hi = lane & b;
#pragma unroll
    for (int q = 0; q < n / 2; ++q) {
      const float send = hi ? w[q] : w[q + n / 2];
      const float keep = hi ? w[q + n / 2] : w[q];
      w[q] = keep + __shfl_xor_sync(0xffffffffu, send, b);
    }
  }
  return w[0];
}

// 255 registers with 2 CTAs per SM; one warp per box with 4 targets per
// lane (168 registers, 3 CTAs per SM) measured 69.4 against 64.2 ms at
// 1,048,576 particles: its 32-lane trees served half the targets each.
__global__ void __launch_bounds__(32 * kNearSymWarps, 2) k_fmm_near_sym(const NearSymArgs p, const AllPairsArgs<float> a,
                                                                   const SceneDesc<float> sc) {
  constexpr int TPT = kNearSymTPT, CH = kNearSymChunk;
  constexpr int TL = 16;    // lanes per target set (a half-warp)
  constexpr int STEP = 4;   // items per sweep step of the warp (2 per half)
  // per warp, two buffers: a unit of a source box's pair items (positions,
  // then dipoles); the next unit is copied into one while the current one is
  // swept from the other
  __shared__ __align__(16) float4 s_pos[kNearSymWarps][2][2 * CH], s_mom[kNearSymWarps][2][2 * CH];
  if (p.done && *p.done != 0.0) return;
  const FmmLevel& lv = p.lv;
  const int lane = threadIdx.x & 31;
  const int w = threadIdx.x >> 5;
  const int tl = lane & (TL - 1);  // slot lane within the target set
  const int half = lane >> 4;      // which items of a step this lane sweeps
  const int64_t c = int64_t(blockIdx.x) * kNearSymWarps + w;
  if (c >= lv.nbox) return;  // warp-uniform; the kernel has no block barrier
  const int32_t n = p.cnt[c];
  if (n == 0) return;
  const int ix = int(c % lv.nx), iy = int((c / lv.nx) % lv.ny), iz = int(c / (int64_t(lv.nx) * lv.ny));
  const int32_t st0 = p.start[c];
  const float near2 = sc.pc.near2_force;
  const float kk = float(kForceK);
  const PairItems::Item zero_item{{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
  // Every lane copies its share of a unit and commits one group per unit
  // (possibly empty), so the lanes' group counts stay in step.
  auto stage = [&](const NearUnit& u, int buf) {
    if (u.plane >= 0) {
      const float4* sp = p.pos2s + u.sb + 2 * u.cs;
      const float4* sm = p.mom2s + u.sb + 2 * u.cs;
      for (int k = lane; k < 2 * u.cn; k += 32) {
        cp_async16(&s_pos[w][buf][k], sp + k);
        cp_async16(&s_mom[w][buf][k], sm + k);
      }
    }
    cp_async_commit();
  };
  for (int t0 = 0; t0 < n; t0 += TL * TPT) {
    float2 tx[TPT], ty[TPT], tz[TPT], tmx[TPT], tmy[TPT], tmz[TPT];
    float2 acc[TPT][3];
#pragma unroll
    for (int t = 0; t < TPT; ++t) {
      const int li = t0 + t * TL + tl;
      const bool live = li < n;
      const int32_t i = p.perm[st0 + (live ? li : 0)];
      const float4 q = a.tpos[i];
      const float4 wm = live ? a.tmom[i] : make_float4(0.f, 0.f, 0.f, 0.f);  // a dead slot adds nothing to sources
      tx[t] = f2_dup(q.x);
      ty[t] = f2_dup(q.y);
      tz[t] = f2_dup(q.z);
      tmx[t] = f2_dup(wm.x);
      tmy[t] = f2_dup(wm.y);
      tmz[t] = f2_dup(wm.z);
      acc[t][0] = acc[t][1] = acc[t][2] = make_float2(0.f, 0.f);
    }
    NearCursor cur{0, 0, 0, 0, 0, 0};
    if (p.n_hrows > 0) {
      const int4 h0 = p.hrows[0];
      cur.dx = (h0.y == 0 && h0.z == 0) ? 1 : -h0.x;
    }
    NearUnit u = near_next(cur, p, ix, iy, iz);
    int buf = 0;
    __syncwarp();  // the previous round's reads of both buffers are done
    stage(u, 0);
    {  // the box's own pairs, target side only (the first unit's copy is in flight)
      const float4* sp = p.pos2s + st0;
      const float4* sm = p.mom2s + st0;
      const int ni = (n + 1) >> 1;
      for (int j = half; j < ni; j += 2) {
        const PairItems::Item it = PairItems::load_item(sp, sm, j);
        float2 src[3] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
#pragma unroll
        for (int t = 0; t < TPT; ++t) sym_force_pair2(tx[t], ty[t], tz[t], tmx[t], tmy[t], tmz[t], it, near2, acc[t], src);
      }
    }
    while (u.plane >= 0) {
      const NearUnit nxt = near_next(cur, p, ix, iy, iz);
      stage(nxt, buf ^ 1);
      cp_async_wait<1>();  // this lane's copies of unit u have landed
      __syncwarp();        // and every lane's
      const float4* wpos = s_pos[w][buf];
      const float4* wmom = s_mom[w][buf];
      float* plane = p.part + int64_t(u.plane) * 3 * p.n_slots;
      const int cn = u.cn;
      // Past the unit's last item: a zero dipole at the origin, nothing on either side.
      for (int j0 = 0; j0 < cn; j0 += STEP) {
        const int jb = j0 + 2 * half;  // this lane's first item of the step
        float v[16];
#pragma unroll
        for (int q = 0; q < 16; ++q) v[q] = 0.f;
#pragma unroll
        for (int q2 = 0; q2 < 2; ++q2) {
          const PairItems::Item it = (jb + q2 < cn) ? PairItems::load_item(wpos, wmom, jb + q2) : zero_item;
          float2 src[3] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
#pragma unroll
          for (int t = 0; t < TPT; ++t) sym_force_pair2(tx[t], ty[t], tz[t], tmx[t], tmy[t], tmz[t], it, near2, acc[t], src);
#pragma unroll
          for (int k = 0; k < 3; ++k) {
            v[q2 * 6 + 2 * k] = src[k].x;
            v[q2 * 6 + 2 * k + 1] = src[k].y;
          }
        }
        // value kv: item jb + kv / 6, component (kv % 6) / 2, source kv % 2
        const float wr = half_reduce_scatter<16>(v, lane);
        const int kv = tl;
        if (kv < 12) {
          const int jl = jb + kv / 6, rem = kv % 6;
          if (jl < cn) {
            float* dst = plane + int64_t(rem >> 1) * p.n_slots + (int64_t(u.sb) + 2 * (u.cs + jl) + (rem & 1));
            const float val = -wr * kk;  // f_ji = -f_ij
            if (t0 == 0) *dst = val;
            else *dst += val;
          }
        }
      }
      __syncwarp();  // every lane is done with buffer buf before it is refilled
      buf ^= 1;
      u = nxt;
    }
    cp_async_wait<0>();
#pragma unroll
    for (int t = 0; t < TPT; ++t) {
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        float s2 = acc[t][k].x + acc[t][k].y;
        s2 += __shfl_xor_sync(0xffffffffu, s2, 16);  // the other half's items
        acc[t][k].x = s2;
      }
      const int li = t0 + t * TL + tl;
      if (li < n && half == 0) {
#pragma unroll
        for (int k = 0; k < 3; ++k) p.part[int64_t(k) * p.n_slots + st0 + li] = acc[t][k].x * kk;
      }
    }
  }
}

unsigned blocks_for(int64_t n, int per = 256, int64_t cap = 65535) {
  int64_t g = (n + per - 1) / per;
  if (g > cap) g = cap;
  return unsigned(g < 1 ? 1 : g);
}

// Taylor coefficients of 1/|R| times gamma!: D_gamma = d^gamma (1/|R|), all
// gamma of degree <= nmax, in graded order.  Recurrence on the coefficients
// T_n = d^n(1/|R|)/n!:  |n| R^2 T_n + (2|n|-1) sum_i R_i T_(n-e_i) + (|n|-1) sum_i T_(n-2e_i) = 0.
void taylor_inv_r(const double R[3], int nmax, std::vector<double>& D) {
  const int N = ncoef(nmax);
  std::vector<double> T(size_t(N), 0.0);
  std::vector<int> mx(static_cast<size_t>(N)), my(static_cast<size_t>(N)), mz(static_cast<size_t>(N));
  const double r2 = R[0] * R[0] + R[1] * R[1] + R[2] * R[2];
  for (int n = 0; n <= nmax; ++n)
    for (int s = 0; s <= n; ++s)
      for (int z = 0; z <= s; ++z) {
        const int x = n - s, y = s - z;
        const int k = gidx(x, y, z);
        mx[size_t(k)] = x;
        my[size_t(k)] = y;
        mz[size_t(k)] = z;
        if (n == 0) {
          T[size_t(k)] = 1.0 / std::sqrt(r2);
          continue;
        }
        const int a[3] = {x, y, z};
        double acc = 0.0;
        for (int i = 0; i < 3; ++i) {
          int b[3] = {x, y, z};
          if (a[i] >= 1) {
            b[i] -= 1;
            acc += double(2 * n - 1) * R[i] * T[size_t(gidx(b[0], b[1], b[2]))];
            b[i] += 1;
          }
          if (a[i] >= 2) {
            b[i] -= 2;
            acc += double(n - 1) * T[size_t(gidx(b[0], b[1], b[2]))];
          }
        }
        T[size_t(k)] = -acc / (double(n) * r2);
      }
  D.assign(size_t(N), 0.0);
  auto fact = [](int v) {
    double f = 1.0;
    for (int i = 2; i <= v; ++i) f *= double(i);
    return f;
  };
  for (int k = 0; k < N; ++k) D[size_t(k)] = T[size_t(k)] * fact(mx[size_t(k)]) * fact(my[size_t(k)]) * fact(mz[size_t(k)]);
}

}  // namespace

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
mf_status Fmm::build(const float4* pos4, int64_t n, const float4* tpos4, int64_t nt, double h, const double* bbox,
                     const FmmConfig& cfg, cudaStream_t st) {
  if (n <= 0) return fail(MF_ERR_INVALID_ARG, "fmm: no particles");
  if (n >= (int64_t(1) << 30) || nt >= (int64_t(1) << 30)) return fail(MF_ERR_INVALID_ARG, "fmm: too many particles");
  if (tpos4 && nt <= 0) return fail(MF_ERR_INVALID_ARG, "fmm: no targets");
  separate_ = tpos4 != nullptr;
  nt_ = separate_ ? nt : n;
  if (cfg.order < 4 || cfg.order > kMaxDegree + 1) return fail(MF_ERR_INVALID_ARG, "fmm: order must be in [4, 10]");
  if (!(cfg.theta > 0.0 && cfg.theta <= 1.0)) return fail(MF_ERR_INVALID_ARG, "fmm: theta must be in (0, 1]");
  if (cfg.leaf_min < 1) return fail(MF_ERR_INVALID_ARG, "fmm: leaf_min must be >= 1");
  cfg_ = cfg;
  degree_ = cfg.order - 1;
  n_ = n;
  const int Q = degree_;
  const int NC = ncoef(Q) - 1;

  // Constant tables (cheap; the module's symbols are per device).
  {
    std::vector<char4> mi(static_cast<size_t>(ncoef(kMaxDegree + 1)));
    for (int d = 0; d <= kMaxDegree + 1; ++d)
      for (int s = 0; s <= d; ++s)
        for (int z = 0; z <= s; ++z) mi[size_t(gidx(d - s, s - z, z))] = make_char4(char(d - s), char(s - z), char(z), 0);
    MF_CUDA_TRY(cudaMemcpyToSymbolAsync(c_mi, mi.data(), mi.size() * sizeof(char4), 0, cudaMemcpyHostToDevice, st));
    float sh[2][kMaxDegree + 2];
    for (int c = 0; c < 2; ++c) {
      const double v = (double(c) - 0.5) / 2.0;
      double f = 1.0;
      for (int j = 0; j < kMaxDegree + 2; ++j) {
        sh[c][j] = float(f);
        f = f * v / double(j + 1);
      }
    }
    MF_CUDA_TRY(cudaMemcpyToSymbolAsync(c_shift, sh, sizeof(sh), 0, cudaMemcpyHostToDevice, st));
  }

  // Box grids.
  double lo[3], ext[3];
  for (int k = 0; k < 3; ++k) {
    lo[k] = bbox[k];
    ext[k] = std::max(0.0, bbox[3 + k] - bbox[k]);
    if (!std::isfinite(lo[k]) || !std::isfinite(ext[k])) return fail(MF_ERR_INVALID_ARG, "fmm: non-finite positions");
  }
  const double emax = std::max({ext[0], ext[1], ext[2]});
  const double S0 = std::max(emax * (1.0 + 1e-5), h * 1e-3);
  for (int k = 0; k < 3; ++k) lo[k] -= 0.25e-5 * S0;
  auto dims_at = [&](int l, int d[3]) {
    const double s = S0 / double(int64_t(1) << l);
    for (int k = 0; k < 3; ++k) {
      int64_t m = int64_t(std::ceil((ext[k] + 0.5e-5 * S0) / s));
      m = std::max<int64_t>(1, std::min<int64_t>(m, int64_t(1) << l));
      d[k] = int(m);
    }
  };
  int L = 2;
  for (int l = 3; l <= kMaxLevel; ++l) {
    int d[3];
    dims_at(l, d);
    const double boxes = double(d[0]) * d[1] * d[2];
    if (double(n) / boxes < double(cfg.leaf_min) || boxes > double(1 << 24)) break;
    L = l;
  }
  lv_.assign(size_t(L + 1), FmmLevel{});
  {
    int d[3];
    dims_at(L, d);
    for (int l = L; l >= 0; --l) {
      FmmLevel& v = lv_[size_t(l)];
      v.nx = d[0];
      v.ny = d[1];
      v.nz = d[2];
      v.nbox = int64_t(d[0]) * d[1] * d[2];
      v.side = float(S0 / double(int64_t(1) << l));
      v.ox = float(lo[0]);
      v.oy = float(lo[1]);
      v.oz = float(lo[2]);
      for (int k = 0; k < 3; ++k) d[k] = (d[k] + 1) / 2;
    }
    int64_t off = 0;
    for (int l = 0; l <= L; ++l) {
      lv_[size_t(l)].box_off = off;
      off += lv_[size_t(l)].nbox;
    }
  }
  const FmmLevel& leaf = lv_[size_t(L)];
  const int64_t nbox_total = leaf.box_off + leaf.nbox;
  const int64_t ncell = leaf.nbox;

  // Bin.
  MF_TRY(occ_.reserve_slack(size_t(nbox_total) * sizeof(int32_t)));
  int32_t* occ = occ_.as<int32_t>();
  int32_t* cnt = occ + leaf.box_off;
  MF_TRY(cell_of_.reserve(size_t(n) * sizeof(int32_t)));
  MF_TRY(start_.reserve_slack(size_t(ncell + 1) * sizeof(int32_t)));
  MF_TRY(cursor_.reserve_slack(size_t(ncell + 1) * sizeof(int32_t)));
  MF_TRY(perm_tmp_.reserve_slack(size_t(n + ncell + 2) * sizeof(int32_t)));
  MF_TRY(perm_.reserve_slack(size_t(n + ncell + 2) * sizeof(int32_t)));
  MF_CUDA_TRY(cudaMemsetAsync(cnt, 0, size_t(ncell) * sizeof(int32_t), st));
  k_fmm_count<<<blocks_for(n), 256, 0, st>>>(pos4, n, leaf, cell_of_.as<int32_t>(), cnt);
  k_fmm_scan<<<1, 1024, 0, st>>>(cnt, ncell, start_.as<int32_t>());
  MF_CUDA_TRY(cudaMemcpyAsync(cursor_.ptr, start_.ptr, size_t(ncell) * sizeof(int32_t), cudaMemcpyDeviceToDevice, st));
  k_fmm_scatter<<<blocks_for(n), 256, 0, st>>>(cell_of_.as<int32_t>(), n, cursor_.as<int32_t>(),
                                                perm_tmp_.as<int32_t>());
  k_fmm_sort<<<blocks_for(ncell * 32), 256, 0, st>>>(start_.as<int32_t>(), cnt, ncell, perm_tmp_.as<int32_t>(),
                                                      perm_.as<int32_t>());
  for (int l = L - 1; l >= 0; --l)
    k_fmm_occ_up<<<blocks_for(lv_[size_t(l)].nbox), 256, 0, st>>>(lv_[size_t(l + 1)], lv_[size_t(l)], occ);
  MF_CUDA_TRY(cudaGetLastError());
  // Separate targets: their own binning into the same leaf boxes (lists in
  // increasing index, padded like the sources), and their own occupancy.
  if (separate_) {
    MF_TRY(tocc_.reserve_slack(size_t(nbox_total) * sizeof(int32_t)));
    int32_t* tocc = tocc_.as<int32_t>();
    int32_t* tcnt = tocc + leaf.box_off;
    MF_TRY(tcell_of_.reserve(size_t(nt) * sizeof(int32_t)));
    MF_TRY(tstart_.reserve_slack(size_t(ncell + 1) * sizeof(int32_t)));
    MF_TRY(tcursor_.reserve_slack(size_t(ncell + 1) * sizeof(int32_t)));
    MF_TRY(tperm_tmp_.reserve_slack(size_t(nt + ncell + 2) * sizeof(int32_t)));
    MF_TRY(tperm_.reserve_slack(size_t(nt + ncell + 2) * sizeof(int32_t)));
    MF_CUDA_TRY(cudaMemsetAsync(tcnt, 0, size_t(ncell) * sizeof(int32_t), st));
    k_fmm_count<<<blocks_for(nt), 256, 0, st>>>(tpos4, nt, leaf, tcell_of_.as<int32_t>(), tcnt);
    k_fmm_scan<<<1, 1024, 0, st>>>(tcnt, ncell, tstart_.as<int32_t>());
    MF_CUDA_TRY(cudaMemcpyAsync(tcursor_.ptr, tstart_.ptr, size_t(ncell) * sizeof(int32_t), cudaMemcpyDeviceToDevice,
                                st));
    k_fmm_scatter<<<blocks_for(nt), 256, 0, st>>>(tcell_of_.as<int32_t>(), nt, tcursor_.as<int32_t>(),
                                                   tperm_tmp_.as<int32_t>());
    k_fmm_sort<<<blocks_for(ncell * 32), 256, 0, st>>>(tstart_.as<int32_t>(), tcnt, ncell, tperm_tmp_.as<int32_t>(),
                                                        tperm_.as<int32_t>());
    for (int l = L - 1; l >= 0; --l)
      k_fmm_occ_up<<<blocks_for(lv_[size_t(l)].nbox), 256, 0, st>>>(lv_[size_t(l + 1)], lv_[size_t(l)], tocc);
    MF_CUDA_TRY(cudaGetLastError());
  }
  // Slots: every box padded to an even count, so at most n + ncell; the
  // kernels read the exact count (start[ncell]) on the device.
  n_slots_ = n + ncell + 1;
  MF_TRY(pos2s_.reserve_slack(size_t(n_slots_ + 2) * sizeof(float4)));
  MF_TRY(mom2s_.reserve_slack(size_t(n_slots_ + 2) * sizeof(float4)));
  k_fmm_gather_pairs<<<blocks_for(n_slots_ / 2), 256, 0, st>>>(perm_.as<int32_t>(), pos4, start_.as<int32_t>() + ncell,
                                                                pos2s_.as<float4>(), 1, nullptr);
  MF_CUDA_TRY(cudaGetLastError());

  // Acceptance: box pairs of one level at centre offset d (box units) are far
  // when theta |d| > r1 + r2 (the box radii, FMMOptions.hpp:56-78) and the gap
  // |d| - (r1 + r2) exceeds the near radius 4h.
  const double rnear = 4.0 * h * (1.0 + 1e-4);
  const double r12 = std::sqrt(3.0);
  auto far = [&](int l, int dx, int dy, int dz) {
    if (l <= 0) return false;
    const double s = double(lv_[size_t(l)].side);
    const double r0 = std::sqrt(double(dx) * dx + double(dy) * dy + double(dz) * dz);
    return cfg.theta * r0 > r12 && (r0 - r12) * s > rnear;
  };
  auto fdiv = [](int a, int b) { return (a >= 0) ? a / b : -((-a + b - 1) / b); };
  std::map<std::tuple<int, int, int>, int> did;
  std::vector<int4> list;
  list_off_.assign(size_t(8 * (L + 1)), 0);
  list_cnt_.assign(size_t(8 * (L + 1)), 0);
  for (int l = 2; l <= L; ++l) {
    const FmmLevel& v = lv_[size_t(l)];
    // Parent offsets that are not accepted are bounded by this radius.
    const double sp = 2.0 * double(v.side);
    const int Dm = int(std::ceil(std::max(r12 / cfg.theta, rnear / sp + r12))) + 1;
    const int R = 2 * Dm + 2;
    for (int cls = 0; cls < 8; ++cls) {
      const int c[3] = {cls & 1, (cls >> 1) & 1, cls >> 2};
      list_off_[size_t(8 * l + cls)] = int64_t(list.size());
      const int Rx = std::min(R, v.nx - 1), Ry = std::min(R, v.ny - 1), Rz = std::min(R, v.nz - 1);
      for (int dz = -Rz; dz <= Rz; ++dz)
        for (int dy = -Ry; dy <= Ry; ++dy)
          for (int dx = -Rx; dx <= Rx; ++dx) {
            if (!far(l, dx, dy, dz)) continue;
            const int d[3] = {dx, dy, dz};
            int D[3];
            for (int k = 0; k < 3; ++k) D[k] = -fdiv(c[k] - d[k], 2);
            if (far(l - 1, D[0], D[1], D[2])) continue;
            auto key = std::make_tuple(dx, dy, dz);
            auto it = did.find(key);
            int id;
            if (it == did.end()) {
              id = int(did.size());
              did.emplace(key, id);
            } else {
              id = it->second;
            }
            list.push_back(make_int4(dx, dy, dz, id));
          }
      list_cnt_[size_t(8 * l + cls)] = int64_t(list.size()) - list_off_[size_t(8 * l + cls)];
    }
  }
  // Near rows of the leaf level: for each (dy, dz), x offsets |dx| <= w.
  std::vector<int4> rows;
  {
    const int R = int(std::ceil(std::max(r12 / cfg.theta, rnear / double(leaf.side) + r12))) + 1;
    const int Rx = std::min(R, leaf.nx - 1), Ry = std::min(R, leaf.ny - 1), Rz = std::min(R, leaf.nz - 1);
    for (int dz = -Rz; dz <= Rz; ++dz)
      for (int dy = -Ry; dy <= Ry; ++dy) {
        if (far(L, 0, dy, dz)) continue;
        int w = 0;
        while (w + 1 <= Rx && !far(L, w + 1, dy, dz)) ++w;
        rows.push_back(make_int4(w, dy, dz, 0));
      }
  }
  n_rows_ = int(rows.size());
  // Half stencil for the near field once per unordered box pair: rows with
  // dz > 0, or dz = 0 and dy > 0 (x offsets -w..w), and the centre row (x
  // offsets 1..w).  w of a half row holds the box offsets before it; its
  // offsets dx take planes 1 + w_before + (dx + w) (centre: dx - 1).
  std::vector<int4> hrows;
  n_off_ = 0;
  for (const int4& r : rows) {
    if (r.z > 0 || (r.z == 0 && r.y > 0)) {
      hrows.push_back(make_int4(r.x, r.y, r.z, n_off_));
      n_off_ += 2 * r.x + 1;
    } else if (r.y == 0 && r.z == 0 && r.x > 0) {
      hrows.push_back(make_int4(r.x, 0, 0, n_off_));
      n_off_ += r.x;
    }
  }
  n_hrows_ = int(hrows.size());
  // Interaction lists, rows and the derivative table are uploaded only when
  // they changed (positions that move a little keep the same grid shape).
  // Uploads go through pinned staging that stays alive until the next build.
  const int NG = ncoef(Q + 1);
  std::vector<int32_t> dkey;
  dkey.reserve(did.size() * 3 + 1);
  dkey.push_back(Q);
  for (const auto& kv : did) {
    dkey.push_back(std::get<0>(kv.first));
    dkey.push_back(std::get<1>(kv.first));
    dkey.push_back(std::get<2>(kv.first));
  }
  const bool same_lists = (list == host_list_) && (rows == host_rows_);
  const bool same_d = (dkey == host_dkey_);
  if (!same_d) {
    // Kernels of earlier products may still read the old tables: the
    // uploads are ordered on the stream, from host copies kept as members.
    MF_CUDA_TRY(cudaStreamSynchronize(st));
    host_dt_.assign(did.size() * size_t(NG), 0.f);
    std::vector<double> D;
    for (const auto& kv : did) {
      const double R[3] = {double(std::get<0>(kv.first)), double(std::get<1>(kv.first)), double(std::get<2>(kv.first))};
      taylor_inv_r(R, Q + 1, D);
      for (int g = 0; g < NG; ++g) host_dt_[size_t(kv.second) * NG + g] = float(D[size_t(g)]);
    }
    MF_TRY(dtab_.reserve_slack(std::max<size_t>(1, host_dt_.size()) * sizeof(float)));
    if (!host_dt_.empty())
      MF_CUDA_TRY(cudaMemcpyAsync(dtab_.ptr, host_dt_.data(), host_dt_.size() * sizeof(float), cudaMemcpyHostToDevice, st));
    host_dkey_ = dkey;
  }
  if (!same_lists) {
    MF_CUDA_TRY(cudaStreamSynchronize(st));
    host_list_ = std::move(list);
    host_rows_ = std::move(rows);
    host_hrows_ = std::move(hrows);
    host_lofs_ = list_off_;
    host_lofs_.insert(host_lofs_.end(), list_cnt_.begin(), list_cnt_.end());
    MF_TRY(lists_.reserve_slack(std::max<size_t>(1, host_list_.size()) * sizeof(int4)));
    MF_TRY(rows_.reserve_slack(std::max<size_t>(1, host_rows_.size()) * sizeof(int4)));
    MF_TRY(hrows_.reserve_slack(std::max<size_t>(1, host_hrows_.size()) * sizeof(int4)));
    MF_TRY(lofs_.reserve_slack(host_lofs_.size() * sizeof(int64_t)));
    if (!host_list_.empty())
      MF_CUDA_TRY(cudaMemcpyAsync(lists_.ptr, host_list_.data(), host_list_.size() * sizeof(int4),
                                  cudaMemcpyHostToDevice, st));
    if (!host_rows_.empty())
      MF_CUDA_TRY(cudaMemcpyAsync(rows_.ptr, host_rows_.data(), host_rows_.size() * sizeof(int4),
                                  cudaMemcpyHostToDevice, st));
    if (!host_hrows_.empty())
      MF_CUDA_TRY(cudaMemcpyAsync(hrows_.ptr, host_hrows_.data(), host_hrows_.size() * sizeof(int4),
                                  cudaMemcpyHostToDevice, st));
    MF_CUDA_TRY(cudaMemcpyAsync(lofs_.ptr, host_lofs_.data(), host_lofs_.size() * sizeof(int64_t),
                                cudaMemcpyHostToDevice, st));
  }

  // Coefficients and the M2L split per level.
  const int sms = device_sms(current_device());
  chunks_.assign(size_t(L + 1), 1);
  int64_t lpart = 1;
  for (int l = 2; l <= L; ++l) {
    const FmmLevel& v = lv_[size_t(l)];
    const int64_t per = ((int64_t((v.nx + 1) / 2) * ((v.ny + 1) / 2) * ((v.nz + 1) / 2)) + 31) / 32 * 32;
    int64_t ch = (int64_t(sms) * 1024 + 8 * per - 1) / (8 * per);
    int64_t maxcnt = 1;
    for (int cls = 0; cls < 8; ++cls) maxcnt = std::max(maxcnt, list_cnt_[size_t(8 * l + cls)]);
    ch = std::max<int64_t>(1, std::min<int64_t>({ch, 16, maxcnt}));
    chunks_[size_t(l)] = int32_t(ch);
    lpart = std::max(lpart, ch * NC * v.nbox);
  }
  MF_TRY(mcoef_.reserve_slack(size_t(NC) * size_t(nbox_total) * sizeof(float)));
  MF_TRY(lcoef_.reserve_slack(size_t(NC) * size_t(nbox_total) * sizeof(float)));
  MF_TRY(lpart_.reserve_slack(size_t(lpart) * sizeof(float)));

  // Statistics, counted on the device and read back lazily (stats()).
  MF_TRY(stat_.reserve(5 * sizeof(unsigned long long)));
  MF_CUDA_TRY(cudaMemsetAsync(stat_.ptr, 0, 5 * sizeof(unsigned long long), st));
  const int32_t* tocc_all = separate_ ? tocc_.as<int32_t>() : occ;
  k_fmm_p2p_stats<<<blocks_for(ncell), 256, 0, st>>>(leaf, cnt, tocc_all + leaf.box_off, rows_.as<int4>(), n_rows_,
                                                      stat_.as<unsigned long long>());
  for (int l = 2; l <= L; ++l)
    k_fmm_m2l_stats<<<blocks_for(lv_[size_t(l)].nbox * 32), 256, 0, st>>>(
        lv_[size_t(l)], occ, tocc_all, lists_.as<int4>(), lofs_.as<int64_t>() + 8 * l,
        lofs_.as<int64_t>() + list_off_.size() + 8 * l, stat_.as<unsigned long long>());
  MF_CUDA_TRY(cudaGetLastError());
  if (!hstat_) MF_CUDA_TRY(cudaMallocHost(&hstat_, 5 * sizeof(unsigned long long)));
  if (!stat_ev_) MF_CUDA_TRY(cudaEventCreateWithFlags(&stat_ev_, cudaEventDisableTiming));
  MF_CUDA_TRY(cudaMemcpyAsync(hstat_, stat_.ptr, 5 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
  MF_CUDA_TRY(cudaEventRecord(stat_ev_, st));
  stat_pending_ = true;
  stats_ = FmmStats{};
  stats_.levels = L + 1;
  stats_.leaf_level = L;
  stats_.degree = Q;
  stats_.leaf_boxes = ncell;
  stats_.near_rows = n_rows_;
  return MF_OK;
}

const FmmStats& Fmm::stats() {
  if (stat_pending_ && stat_ev_ && cudaEventSynchronize(stat_ev_) == cudaSuccess) {
    stats_.p2p_pairs = double(hstat_[0]);
    stats_.max_leaf = int32_t(hstat_[1]);
    stats_.m2l_per_product = double(hstat_[2]);
    stats_.occupied_leaves = int64_t(hstat_[3]);
    stats_.p2p_self_pairs = double(hstat_[4]);
    stat_pending_ = false;
  }
  return stats_;
}

Fmm::~Fmm() {
  if (hstat_) pinned_free(hstat_);
  if (stat_ev_) cudaEventDestroy(stat_ev_);
}

mf_status Fmm::product(int kind, const float4* pos4, const float4* smom, const AllPairsArgs<float>& a,
                       const SceneDesc<float>& sc, cudaStream_t st, const double* done, cudaEvent_t* marks,
                       bool sym_near) {
  if (kind < 0 || kind > 2) return fail(MF_ERR_INVALID_ARG, "fmm: unknown product kind");
  switch (degree_) {
    case 3: return product_q<3>(kind, pos4, smom, a, sc, st, done, marks, sym_near);
    case 4: return product_q<4>(kind, pos4, smom, a, sc, st, done, marks, sym_near);
    case 5: return product_q<5>(kind, pos4, smom, a, sc, st, done, marks, sym_near);
    case 6: return product_q<6>(kind, pos4, smom, a, sc, st, done, marks, sym_near);
    case 7: return product_q<7>(kind, pos4, smom, a, sc, st, done, marks, sym_near);
    case 8: return product_q<8>(kind, pos4, smom, a, sc, st, done, marks, sym_near);
    case 9:
      if (kind == 0) return fail(MF_ERR_INVALID_ARG, "fmm: order 10 is for the force products only");
      return product_q<9>(kind, pos4, smom, a, sc, st, done, marks, sym_near);
    default: return fail(MF_ERR_INVALID_ARG, "fmm: unsupported degree");
  }
}

namespace {
// M2L launches of one level, split by local degree so the multipole and the
// accumulators stay in registers.  hess: the product needs only the Hessian
// of the local expansion (the Kelvin force, the force tensor), which no local
// of degree 1 reaches (L2L maps degree >= 2 only from degree >= 2, and L2P of
// the Hessian reads degree >= 2), so the degree-1 locals are not computed.
template <int Q>
struct M2LVariants;
template <>
struct M2LVariants<3> {
  static void launch(const M2LArgs& p, unsigned g, cudaStream_t st, int* n, bool hess) {
    if (hess) k_fmm_m2l<3, 2, 3><<<g, 128, 0, st>>>(p);
    else k_fmm_m2l<3, 1, 3><<<g, 128, 0, st>>>(p);
    *n += 1;
  }
};
template <>
struct M2LVariants<4> {
  static void launch(const M2LArgs& p, unsigned g, cudaStream_t st, int* n, bool hess) {
    if (hess) k_fmm_m2l<4, 2, 4><<<g, 128, 0, st>>>(p);
    else k_fmm_m2l<4, 1, 4><<<g, 128, 0, st>>>(p);
    *n += 1;
  }
};
template <>
struct M2LVariants<5> {
  static void launch(const M2LArgs& p, unsigned g, cudaStream_t st, int* n, bool hess) {
    if (hess) k_fmm_m2l<5, 2, 5><<<g, 128, 0, st>>>(p);
    else k_fmm_m2l<5, 1, 5><<<g, 128, 0, st>>>(p);
    *n += 1;
  }
};
template <>
struct M2LVariants<6> {
  static void launch(const M2LArgs& p, unsigned g, cudaStream_t st, int* n, bool hess) {
    if (hess) k_fmm_m2l<6, 2, 2><<<g, 128, 0, st>>>(p);
    else k_fmm_m2l<6, 1, 2><<<g, 128, 0, st>>>(p);
    k_fmm_m2l<6, 3, 6><<<g, 128, 0, st>>>(p);
    *n += 2;
  }
};
template <>
struct M2LVariants<7> {
  static void launch(const M2LArgs& p, unsigned g, cudaStream_t st, int* n, bool hess) {
    if (hess) k_fmm_m2l<7, 2, 3><<<g, 128, 0, st>>>(p);
    else k_fmm_m2l<7, 1, 3><<<g, 128, 0, st>>>(p);
    k_fmm_m2l<7, 4, 7><<<g, 128, 0, st>>>(p);
    *n += 2;
  }
};
template <>
struct M2LVariants<8> {
  static void launch(const M2LArgs& p, unsigned g, cudaStream_t st, int* n, bool hess) {
    if (hess) {
      k_fmm_m2l<8, 2, 3><<<g, 128, 0, st>>>(p);
      k_fmm_m2l<8, 4, 5><<<g, 128, 0, st>>>(p);
      k_fmm_m2l<8, 6, 8><<<g, 128, 0, st>>>(p);
    } else {
      k_fmm_m2l<8, 1, 2><<<g, 128, 0, st>>>(p);
      k_fmm_m2l<8, 3, 4><<<g, 128, 0, st>>>(p);
      k_fmm_m2l<8, 5, 8><<<g, 128, 0, st>>>(p);
    }
    *n += 3;
  }
};
template <>
struct M2LVariants<9> {
  // The force products only (Fmm::product refuses a field product at degree 9).
  static void launch(const M2LArgs& p, unsigned g, cudaStream_t st, int* n, bool hess) {
    if (!hess) return;
    k_fmm_m2l<9, 2, 3><<<g, 128, 0, st>>>(p);
    k_fmm_m2l<9, 4, 5><<<g, 128, 0, st>>>(p);
    k_fmm_m2l<9, 6, 7><<<g, 128, 0, st>>>(p);
    k_fmm_m2l<9, 8, 9><<<g, 128, 0, st>>>(p);
    *n += 4;
  }
};
// One CTA of 128 threads per leaf box, 256-source stages, also for small
// boxes: 64 threads with 128-source stages measured slower at 262,144
// particles (boxes of <= 40: near field 3.9 against 2.7 ms for the field,
// 11.3 against 7.3 for the force): the step and barrier count per box doubles.
template <int Q, int kKind, bool kParts>
void launch_p2p(unsigned grid, cudaStream_t st, const P2PArgs& pp, const AllPairsArgs<float>& a,
                const SceneDesc<float>& sc) {
  k_fmm_p2p<Q, kKind, kParts, 128, 256><<<grid, 128, p2p_smem<256>(), st>>>(pp, a, sc);
}
}  // namespace

template <int Q>
mf_status Fmm::product_q(int kind, const float4* pos4, const float4* smom, const AllPairsArgs<float>& a,
                         const SceneDesc<float>& sc, cudaStream_t st, const double* done, cudaEvent_t* marks,
                         bool sym_near) {
  constexpr int NC = ncoef(Q) - 1;
  const int L = int(lv_.size()) - 1;
  const FmmLevel& leaf = lv_[size_t(L)];
  int32_t* occ = occ_.as<int32_t>();
  const int32_t* cnt = occ + leaf.box_off;
  const int32_t* tocc = separate_ ? tocc_.as<int32_t>() : occ;
  float* M = mcoef_.as<float>();
  float* Lc = lcoef_.as<float>();
  int nl = 0;
  if (marks) MF_CUDA_TRY(cudaEventRecord(marks[0], st));
  k_fmm_gather_pairs<<<blocks_for(n_slots_ / 2), 256, 0, st>>>(perm_.as<int32_t>(), smom, start_.as<int32_t>() + leaf.nbox,
                                                                mom2s_.as<float4>(), 0, done);
  ++nl;
  const int sms = device_sms(current_device());
  k_fmm_p2m<Q><<<blocks_for(leaf.nbox, 1, int64_t(sms) * 16), 128, 0, st>>>(
      leaf, start_.as<int32_t>(), cnt, perm_.as<int32_t>(), pos4, smom, M + leaf.box_off * NC, done);
  ++nl;
  for (int l = L - 1; l >= 2; --l) {
    k_fmm_m2m<Q><<<blocks_for(int64_t(NC) * lv_[size_t(l)].nbox, 256, int64_t(sms) * 32), 256, 0, st>>>(
        lv_[size_t(l + 1)], lv_[size_t(l)], occ, M, done);
    ++nl;
  }
  for (int l = 2; l <= L; ++l) {
    const FmmLevel& v = lv_[size_t(l)];
    M2LArgs p{};
    p.lv = v;
    p.occ = occ;
    p.tocc = tocc;
    p.M = M + v.box_off * NC;
    p.Lp = lpart_.as<float>();
    p.list = lists_.as<int4>();
    p.dtab = dtab_.as<float>();
    for (int cls = 0; cls < 8; ++cls) {
      p.list_off[cls] = list_off_[size_t(8 * l + cls)];
      p.list_cnt[cls] = int32_t(list_cnt_[size_t(8 * l + cls)]);
    }
    p.chunks = chunks_[size_t(l)];
    p.hx = (v.nx + 1) / 2;
    p.hy = (v.ny + 1) / 2;
    p.hz = (v.nz + 1) / 2;
    p.per_class = ((int64_t(p.hx) * p.hy * p.hz) + 31) / 32 * 32;
    p.done = done;
    const int64_t threads = int64_t(p.chunks) * 8 * p.per_class;
    M2LVariants<Q>::launch(p, unsigned((threads + 127) / 128), st, &nl, kind != 0);
    k_fmm_l2l<Q><<<blocks_for(int64_t(NC) * v.nbox, 256, int64_t(sms) * 32), 256, 0, st>>>(
        v, lv_[size_t(l - 1)], l > 2 ? 1 : 0, tocc, lpart_.as<float>(), p.chunks, Lc, done, kind != 0 ? 3 : 0);
    ++nl;
  }
  P2PArgs pp{};
  pp.lv = leaf;
  pp.start = start_.as<int32_t>();
  pp.cnt = cnt;
  pp.perm = perm_.as<int32_t>();
  pp.tstart = separate_ ? tstart_.as<int32_t>() : pp.start;
  pp.tcnt = tocc + leaf.box_off;
  pp.tperm = separate_ ? tperm_.as<int32_t>() : pp.perm;
  pp.pos2s = pos2s_.as<float4>();
  pp.mom2s = mom2s_.as<float4>();
  pp.L = Lc + leaf.box_off * NC;
  pp.rows = rows_.as<int4>();
  pp.n_rows = n_rows_;
  pp.done = done;
  const bool sym = kind == 1 && sym_near && !separate_;
  if (sym) {
    MF_TRY(npart_.reserve_grow(size_t(1 + n_off_) * 3 * size_t(n_slots_) * sizeof(float)));
    pp.hrows = hrows_.as<int4>();
    pp.n_hrows = n_hrows_;
    pp.part = npart_.as<float>();
    pp.n_slots = n_slots_;
  }
  if (leaf.nbox > int64_t(0x7fffffff)) return fail(MF_ERR_INVALID_ARG, "fmm: too many leaf boxes");
  if (marks) {
    MF_CUDA_TRY(cudaEventRecord(marks[1], st));
    MF_CUDA_TRY(cudaEventRecord(marks[2], st));
  }
  if (sym) {
    NearSymArgs ns{};
    ns.lv = leaf;
    ns.start = pp.start;
    ns.cnt = cnt;
    ns.perm = pp.perm;
    ns.pos2s = pp.pos2s;
    ns.mom2s = pp.mom2s;
    ns.hrows = pp.hrows;
    ns.n_hrows = n_hrows_;
    ns.part = npart_.as<float>();
    ns.n_slots = n_slots_;
    ns.done = done;
    k_fmm_near_sym<<<unsigned((leaf.nbox + kNearSymWarps - 1) / kNearSymWarps), 32 * kNearSymWarps, 0, st>>>(ns, a, sc);
    ++nl;
    launch_p2p<Q, 1, true>(unsigned(leaf.nbox), st, pp, a, sc);
  } else if (kind == 1)
    launch_p2p<Q, 1, false>(unsigned(leaf.nbox), st, pp, a, sc);
  else if (kind == 2)
    launch_p2p<Q, 2, false>(unsigned(leaf.nbox), st, pp, a, sc);
  else
    if constexpr (Q <= kMaxFieldDegree) launch_p2p<Q, 0, false>(unsigned(leaf.nbox), st, pp, a, sc);
  ++nl;
  if (marks) MF_CUDA_TRY(cudaEventRecord(marks[3], st));
  launches_ = nl;
  MF_CUDA_TRY(cudaGetLastError());
  return MF_OK;
}

}  // namespace mfgb

// ===========================================================================
// C ABI: an FMM matrix over a source set and a target set
// ===========================================================================
struct mf_fmm {
  int device = 0;
  cudaStream_t st = nullptr;
  mfgb::Fmm fmm;
  // The Hessian product's lists at the force aperture, built on its first
  // call when that aperture is smaller than the field's.
  mfgb::Fmm fmmh;
  bool fmmh_built = false;
  mfgb::FmmConfig cfg;
  double h = 0.0, bbox[6] = {0, 0, 0, 0, 0, 0};
  mfgb::CellList cells;  // over the sources: the near-field correction
  mfgb::Scratch scr;
  mfgb::DevBuf spos, smom, tpos, corr, out4, out9, staging;
  int64_t ns = 0, nt = 0;
  bool same = true;
  mfgb::SceneDesc<float> sc{};
  ~mf_fmm() {
    if (st) {
      cudaStreamSynchronize(st);
      cudaStreamDestroy(st);
    }
  }
};

namespace mfgb {
namespace {
__global__ void k_aos_to_f4(const float* __restrict__ src, int64_t n, float4* __restrict__ dst,
                            int32_t* __restrict__ bad) {
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
    const float x = src[3 * i], y = src[3 * i + 1], z = src[3 * i + 2];
    if (!isfinite(x) || !isfinite(y) || !isfinite(z)) atomicExch(bad, 1);
    dst[i] = make_float4(x, y, z, 0.f);
  }
}
// 9 SoA arrays (k = column * 3 + row) -> [n][9] in the same order per target.
__global__ void k_soa9_to_aos(const float* __restrict__ src, int64_t n, float* __restrict__ dst) {
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
#pragma unroll
    for (int k = 0; k < 9; ++k) dst[9 * i + k] = src[int64_t(k) * n + i];
}
__global__ void k_f4_to_aos(const float4* __restrict__ src, int64_t n, float* __restrict__ dst) {
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
    const float4 v = src[i];
    dst[3 * i] = v.x;
    dst[3 * i + 1] = v.y;
    dst[3 * i + 2] = v.z;
  }
}

// Host AoS float[n][3] -> device float4 records (through `staging`); checks finiteness.
mf_status upload_f4(mf_fmm& f, const float* host, int64_t n, DevBuf& dst) {
  MF_TRY(f.staging.reserve(size_t(3 * n) * sizeof(float) + 16));
  MF_TRY(dst.reserve(size_t(n + 2) * sizeof(float4), false, true));
  int32_t* bad = reinterpret_cast<int32_t*>(f.staging.as<char>() + size_t(3 * n) * sizeof(float));
  MF_CUDA_TRY(cudaMemsetAsync(bad, 0, sizeof(int32_t), f.st));
  MF_CUDA_TRY(cudaMemcpyAsync(f.staging.ptr, host, size_t(3 * n) * sizeof(float), cudaMemcpyHostToDevice, f.st));
  k_aos_to_f4<<<blocks_for(n), 256, 0, f.st>>>(f.staging.as<float>(), n, dst.as<float4>(), bad);
  MF_CUDA_TRY(cudaGetLastError());
  int32_t hb = 0;
  MF_CUDA_TRY(cudaMemcpyAsync(&hb, bad, sizeof(int32_t), cudaMemcpyDeviceToHost, f.st));
  MF_CUDA_TRY(cudaStreamSynchronize(f.st));
  if (hb) return fail(MF_ERR_INVALID_ARG, "non-finite input value");
  return MF_OK;
}

template <class F>
mf_status fguard(mf_fmm* f, F&& fn) {
  if (!f) return fail(MF_ERR_INVALID_ARG, "NULL fmm handle");
  try {
    cudaError_t e = cudaSetDevice(f->device);
    if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
    return fn(*f);
  } catch (const std::bad_alloc&) {
    return fail(MF_ERR_OOM, "host allocation failed");
  } catch (...) {
    return fail(MF_ERR_CUDA, "unexpected exception");
  }
}
}  // namespace
}  // namespace mfgb

using namespace mfgb;

extern "C" {

mf_status mf_fmm_create(const float* sources, int64_t ns, const float* targets, int64_t nt, float h, int32_t order,
                        double theta, int32_t leaf_min, int32_t device, mf_fmm** out) {
  if (!out || !sources || ns <= 0) return fail(MF_ERR_INVALID_ARG, "fmm: no sources");
  *out = nullptr;
  if (targets && nt <= 0) return fail(MF_ERR_INVALID_ARG, "fmm: no targets");
  if (!(h > 0.f) || !std::isfinite(h)) return fail(MF_ERR_INVALID_ARG, "fmm: h must be finite and > 0");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(MF_ERR_UNSUPPORTED, "no CUDA device available");
  if (device < 0 || device >= ndev) return fail(MF_ERR_INVALID_ARG, "bad device ordinal");
  try {
    MF_CUDA_TRY(cudaSetDevice(device));
    std::unique_ptr<mf_fmm> f(new mf_fmm);
    f->device = device;
    MF_CUDA_TRY(cudaStreamCreateWithFlags(&f->st, cudaStreamNonBlocking));
    f->ns = ns;
    f->same = targets == nullptr;
    f->nt = f->same ? ns : nt;
    MF_TRY(upload_f4(*f, sources, ns, f->spos));
    if (!f->same) MF_TRY(upload_f4(*f, targets, nt, f->tpos));
    MF_TRY(f->cells.build(f->spos.as<float4>(), {CellSceneSpec{0, ns, double(h)}}, f->st));
    double bbox[6];
    for (int k = 0; k < 6; ++k) bbox[k] = f->cells.bbox(0)[k];
    if (!f->same)
      for (int64_t i = 0; i < nt; ++i)
        for (int k = 0; k < 3; ++k) {
          bbox[k] = std::min(bbox[k], double(targets[3 * i + k]));
          bbox[3 + k] = std::max(bbox[3 + k], double(targets[3 * i + k]));
        }
    FmmConfig& cfg = f->cfg;
    cfg.order = order;
    cfg.theta = theta;
    cfg.leaf_min = leaf_min;
    f->h = double(h);
    for (int k = 0; k < 6; ++k) f->bbox[k] = bbox[k];
    MF_TRY(f->fmm.build(f->spos.as<float4>(), ns, f->same ? nullptr : f->tpos.as<float4>(), f->nt, double(h), bbox,
                        cfg, f->st));
    MF_TRY(f->corr.reserve(size_t(f->nt + 2) * sizeof(float4), false, true));
    MF_TRY(f->out4.reserve(size_t(f->nt + 2) * sizeof(float4), false, true));
    MF_TRY(f->scr.ensure(0, 0));
    f->sc.pc = make_pair_consts<float>(double(h));
    f->sc.scale = 1.f;
    MF_CUDA_TRY(cudaStreamSynchronize(f->st));
    *out = f.release();
    return MF_OK;
  } catch (const std::bad_alloc&) {
    return fail(MF_ERR_OOM, "host allocation failed");
  }
}

mf_status mf_fmm_destroy(mf_fmm* f) {
  if (!f) return MF_OK;
  cudaSetDevice(f->device);
  delete f;
  return MF_OK;
}

mf_status mf_fmm_field(mf_fmm* f, const float* charges, float* results) {
  return fguard(f, [&](mf_fmm& x) {
    if (!charges || !results) return fail(MF_ERR_INVALID_ARG, "NULL argument");
    MF_TRY(upload_f4(x, charges, x.ns, x.smom));
    const float4* tp = x.same ? x.spos.as<float4>() : x.tpos.as<float4>();
    if (x.same)
      MF_TRY(x.cells.field_correction(x.spos.as<float4>(), x.smom.as<float4>(), x.corr.as<float4>(), x.st));
    else
      MF_TRY(x.cells.field_correction_at(tp, x.nt, x.spos.as<float4>(), x.smom.as<float4>(), x.corr.as<float4>(),
                                         x.st));
    AllPairsArgs<float> a{};
    a.tpos = tp;
    a.corr4 = x.corr.as<float4>();
    a.out4 = x.out4.as<float4>();
    a.err = x.scr.err.as<int32_t>();
    MF_TRY(x.fmm.product(0, x.spos.as<float4>(), x.smom.as<float4>(), a, x.sc, x.st, nullptr));
    MF_TRY(x.staging.reserve(size_t(3 * x.nt) * sizeof(float) + 16));
    k_f4_to_aos<<<blocks_for(x.nt), 256, 0, x.st>>>(x.out4.as<float4>(), x.nt, x.staging.as<float>());
    MF_CUDA_TRY(cudaGetLastError());
    MF_CUDA_TRY(cudaMemcpyAsync(results, x.staging.ptr, size_t(3 * x.nt) * sizeof(float), cudaMemcpyDeviceToHost,
                                x.st));
    MF_CUDA_TRY(cudaStreamSynchronize(x.st));
    return x.scr.check(x.st);
  });
}

mf_status mf_fmm_hessian(mf_fmm* f, const float* charges, float* results9) {
  return fguard(f, [&](mf_fmm& x) {
    if (!charges || !results9) return fail(MF_ERR_INVALID_ARG, "NULL argument");
    MF_TRY(upload_f4(x, charges, x.ns, x.smom));
    const float4* tp = x.same ? x.spos.as<float4>() : x.tpos.as<float4>();
    MF_TRY(x.corr.reserve(size_t(2 * x.nt + 2) * sizeof(float4), false, true));
    MF_TRY(x.cells.tensor_correction_at(tp, x.nt, x.spos.as<float4>(), x.smom.as<float4>(), x.corr.as<float4>(),
                                        x.st));
    MF_TRY(x.out9.reserve(size_t(9 * x.nt) * sizeof(float)));
    AllPairsArgs<float> a{};
    a.tpos = tp;
    a.corr4 = x.corr.as<float4>();
    for (int k = 0; k < 9; ++k) a.out[k] = x.out9.as<float>() + size_t(k) * size_t(x.nt);
    a.err = x.scr.err.as<int32_t>();
    Fmm* fh = &x.fmm;
    if (x.cfg.force_tree()) {
      if (!x.fmmh_built) {
        FmmConfig ct = x.cfg;
        ct.theta = x.cfg.force_theta();
        ct.order = x.cfg.force_order();
        MF_TRY(x.fmmh.build(x.spos.as<float4>(), x.ns, x.same ? nullptr : x.tpos.as<float4>(), x.nt, x.h, x.bbox, ct,
                            x.st));
        x.fmmh_built = true;
      }
      fh = &x.fmmh;
    }
    MF_TRY(fh->product(2, x.spos.as<float4>(), x.smom.as<float4>(), a, x.sc, x.st, nullptr));
    MF_TRY(x.staging.reserve(size_t(9 * x.nt) * sizeof(float) + 16));
    k_soa9_to_aos<<<blocks_for(x.nt), 256, 0, x.st>>>(x.out9.as<float>(), x.nt, x.staging.as<float>());
    MF_CUDA_TRY(cudaGetLastError());
    MF_CUDA_TRY(cudaMemcpyAsync(results9, x.staging.ptr, size_t(9 * x.nt) * sizeof(float), cudaMemcpyDeviceToHost,
                                x.st));
    MF_CUDA_TRY(cudaStreamSynchronize(x.st));
    return x.scr.check(x.st);
  });
}

mf_status mf_fmm_get_stats(mf_fmm* f, mf_fmm_stats* out) {
  return fguard(f, [&](mf_fmm& x) {
    if (!out) return fail(MF_ERR_INVALID_ARG, "NULL");
    *out = mf_fmm_stats{};
    const FmmStats& s = x.fmm.stats();
    out->active = 1;
    out->levels = s.levels;
    out->leaf_level = s.leaf_level;
    out->degree = s.degree;
    out->leaf_boxes = s.leaf_boxes;
    out->occupied_leaves = s.occupied_leaves;
    out->max_leaf = s.max_leaf;
    out->near_rows = s.near_rows;
    out->p2p_pairs = s.p2p_pairs;
    out->m2l_per_product = s.m2l_per_product;
    out->launches_per_product = x.fmm.launches_per_product();
    out->force_active = 1;
    out->theta = x.cfg.theta;
    out->force_theta = x.cfg.force_theta();
    if (x.fmmh_built) {
      out->force_p2p_pairs = x.fmmh.stats().p2p_pairs;
      out->force_m2l_per_product = x.fmmh.stats().m2l_per_product;
    } else if (!x.cfg.force_tree()) {
      out->force_p2p_pairs = s.p2p_pairs;
      out->force_m2l_per_product = s.m2l_per_product;
    }
    return MF_OK;
  });
}

}  // extern "C"
