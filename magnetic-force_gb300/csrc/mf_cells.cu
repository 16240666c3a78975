// mf_cells.cu -- uniform-grid cell lists and the near-field correction pass.
//
// The packed all-pairs loop (FieldF2Body / ForceF2Body) evaluates every pair
// with the far-field form at max(r^2, r_near^2), which is exact beyond the
// near radius (2h for the field, 4h for the force) and merely finite inside
// it.  This pass visits, for each target, only the sources inside that radius
// (through a cell list with cells of edge >= 2h) and adds
//     exact pair term (SPH weights / fitted curves) - clamped far term,
// so the sum of both launches is the reference's kernel over all pairs.
// Near pairs are about 0.4 % (field) and 3 % (force) of all pairs at the
// benchmark densities.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "mf_internal.h"

namespace mfgb {
namespace {

__device__ __forceinline__ int32_t f2ord(float f) {
  const int32_t b = __float_as_int(f);
  return b >= 0 ? b : b ^ 0x7fffffff;
}
__host__ __device__ __forceinline__ float ord2f(int32_t b) {
#ifdef __CUDA_ARCH__
  return __int_as_float(b >= 0 ? b : b ^ 0x7fffffff);
#else
  int32_t v = b >= 0 ? b : b ^ 0x7fffffff;
  float f;
  memcpy(&f, &v, 4);
  return f;
#endif
}

__device__ __forceinline__ int scene_of(const CellGrid* g, int n, int64_t i) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (g[mid].p_off <= i) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

__global__ void k_bbox_init(int32_t* bbox, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < 6 * n) bbox[i] = (i % 6) < 3 ? 0x7fffffff : int32_t(0x80000000);
}

// blockIdx.y = scene; blocks stride over its particles.
__global__ void k_bbox(const float4* __restrict__ pos, const int64_t* __restrict__ ranges, int32_t* bbox) {
  const int s = blockIdx.y;
  const int64_t off = ranges[2 * s], n = ranges[2 * s + 1];
  float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; k < n; k += int64_t(gridDim.x) * blockDim.x) {
    const float4 p = pos[off + k];
    lo[0] = fminf(lo[0], p.x);
    lo[1] = fminf(lo[1], p.y);
    lo[2] = fminf(lo[2], p.z);
    hi[0] = fmaxf(hi[0], p.x);
    hi[1] = fmaxf(hi[1], p.y);
    hi[2] = fmaxf(hi[2], p.z);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      lo[c] = fminf(lo[c], __shfl_down_sync(0xffffffffu, lo[c], o));
      hi[c] = fmaxf(hi[c], __shfl_down_sync(0xffffffffu, hi[c], o));
    }
  if ((threadIdx.x & 31) == 0)
    for (int c = 0; c < 3; ++c) {
      atomicMin(&bbox[6 * s + c], f2ord(lo[c]));
      atomicMax(&bbox[6 * s + 3 + c], f2ord(hi[c]));
    }
}

__device__ __forceinline__ void cell_coords(const CellGrid& g, float x, float y, float z, int& ix, int& iy,
                                            int& iz) {
  ix = min(max(int((x - g.ox) * g.inv_cs), 0), g.nx - 1);
  iy = min(max(int((y - g.oy) * g.inv_cs), 0), g.ny - 1);
  iz = min(max(int((z - g.oz) * g.inv_cs), 0), g.nz - 1);
}

__global__ void k_count(const float4* __restrict__ pos, const CellGrid* __restrict__ grids, int n_scenes,
                        int64_t n_total, int32_t* __restrict__ counts, int32_t* __restrict__ cell_of) {
  for (int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; k < n_total;
       k += int64_t(gridDim.x) * blockDim.x) {
    // k enumerates the scenes' particles back to back; map it to a particle index.
    int lo = 0, hi = n_scenes - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (grids[mid].k_off <= k) lo = mid;
      else hi = mid - 1;
    }
    const CellGrid& g = grids[lo];
    const int64_t i = g.p_off + (k - g.k_off);
    const float4 p = pos[i];
    int ix, iy, iz;
    cell_coords(g, p.x, p.y, p.z, ix, iy, iz);
    const int64_t c = g.cell_off + (int64_t(iz) * g.ny + iy) * g.nx + ix;
    cell_of[k] = int32_t(c);
    atomicAdd(&counts[c], 1);
  }
}

// Exclusive scan of counts[0..n) into start[0..n], in three launches:
// per-tile sums, a scan of the tile sums, and each tile's scan plus its
// offset.  Tiles are kScanTile consecutive counts; integer sums, so the
// result does not depend on the split.
constexpr int kScanThreads = 256, kScanPer = 16, kScanTile = kScanThreads * kScanPer;

// Exclusive prefix of v over the block (blockDim.x == kScanThreads); *total
// gets the block's sum.  Uses `ws` (kScanThreads / 32 ints of shared memory).
__device__ __forceinline__ int32_t block_exclusive_scan(int32_t v, int32_t* ws, int32_t* total) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  constexpr int kW = kScanThreads / 32;
  int32_t inc = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int32_t t = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += t;
  }
  __syncthreads();  // ws is free (an earlier call may still read it)
  if (lane == 31) ws[w] = inc;
  __syncthreads();
  if (w == 0) {
    const int32_t x = lane < kW ? ws[lane] : 0;
    int32_t xi = x;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int32_t t = __shfl_up_sync(0xffffffffu, xi, o);
      if (lane >= o) xi += t;
    }
    if (lane < kW) ws[lane] = xi - x;
    if (lane == kW - 1) ws[kW] = xi;
  }
  __syncthreads();
  *total = ws[kW];
  return inc - v + ws[w];
}

__global__ void __launch_bounds__(kScanThreads) k_scan_tiles(const int32_t* __restrict__ counts, int64_t n,
                                                             int32_t* __restrict__ tile_sum) {
  __shared__ int32_t ws[kScanThreads / 32 + 1];
  const int64_t base = int64_t(blockIdx.x) * kScanTile;
  int32_t s = 0;
#pragma unroll
  for (int k = 0; k < kScanPer; ++k) {
    const int64_t i = base + int64_t(k) * kScanThreads + threadIdx.x;
    if (i < n) s += counts[i];
  }
  int32_t total;
  block_exclusive_scan(s, ws, &total);
  if (threadIdx.x == 0) tile_sum[blockIdx.x] = total;
}

// One block: tile sums -> exclusive tile offsets (in place); start[n] = total.
__global__ void __launch_bounds__(kScanThreads) k_scan_tile_sums(int32_t* __restrict__ tile_sum, int64_t n_tiles,
                                                                 int32_t* __restrict__ start, int64_t n) {
  __shared__ int32_t ws[kScanThreads / 32 + 1];
  int32_t run = 0;
  for (int64_t b0 = 0; b0 < n_tiles; b0 += kScanThreads) {
    const int64_t b = b0 + threadIdx.x;
    const int32_t v = b < n_tiles ? tile_sum[b] : 0;
    int32_t total;
    const int32_t ex = block_exclusive_scan(v, ws, &total);
    if (b < n_tiles) tile_sum[b] = run + ex;
    run += total;
  }
  if (threadIdx.x == 0) start[n] = run;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_apply(const int32_t* __restrict__ counts, int64_t n,
                                                             const int32_t* __restrict__ tile_off,
                                                             int32_t* __restrict__ start) {
  __shared__ int32_t ws[kScanThreads / 32 + 1];
  const int64_t base = int64_t(blockIdx.x) * kScanTile + int64_t(threadIdx.x) * kScanPer;
  int32_t c[kScanPer];
  int32_t s = 0;
#pragma unroll
  for (int k = 0; k < kScanPer; ++k) {
    c[k] = base + k < n ? counts[base + k] : 0;
    s += c[k];
  }
  int32_t total;
  int32_t run = tile_off[blockIdx.x] + block_exclusive_scan(s, ws, &total);
#pragma unroll
  for (int k = 0; k < kScanPer; ++k) {
    if (base + k < n) start[base + k] = run;
    run += c[k];
  }
}

__global__ void k_scatter(const CellGrid* __restrict__ grids, int n_scenes, int64_t n_total,
                          const int32_t* __restrict__ cell_of, int32_t* __restrict__ cursor,
                          int32_t* __restrict__ perm) {
  for (int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; k < n_total;
       k += int64_t(gridDim.x) * blockDim.x) {
    int lo = 0, hi = n_scenes - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (grids[mid].k_off <= k) lo = mid;
      else hi = mid - 1;
    }
    const int64_t i = grids[lo].p_off + (k - grids[lo].k_off);
    const int32_t slot = atomicAdd(&cursor[cell_of[k]], 1);
    perm[slot] = int32_t(i);
  }
}

// Each cell's list in increasing particle index: one warp per cell places
// every entry at its rank (entries are distinct), from the scattered list
// `in` into `out`.
__global__ void k_sort_cells(const int32_t* __restrict__ start, int64_t n_cells, const int32_t* __restrict__ in,
                             int32_t* __restrict__ out) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = int64_t(gridDim.x) * (blockDim.x >> 5);
  for (int64_t c = int64_t(blockIdx.x) * (blockDim.x >> 5) + (threadIdx.x >> 5); c < n_cells; c += warps) {
    const int32_t b = start[c], m = start[c + 1] - b;
    for (int32_t k = lane; k < m; k += 32) {
      const int32_t v = in[b + k];
      int32_t rank = 0;
      for (int32_t l = 0; l < m; ++l) rank += in[b + l] < v;
      out[b + rank] = v;
    }
  }
}

__constant__ float c_fit_tbl[40] = MF_FITTED_CURVE_TABLE;

// The binned particles in cell order (positions and the product's dipoles),
// so the correction reads each row of cells as one contiguous range.
__global__ void k_gather_sorted(const int32_t* __restrict__ perm, const float4* __restrict__ pos,
                                const float4* __restrict__ mom, int64_t n, float4* __restrict__ spos,
                                float4* __restrict__ smom, const int32_t* __restrict__ done_count, int done_total) {
  if (done_count && *done_count >= done_total) return;
  for (int64_t q = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; q < n; q += int64_t(gridDim.x) * blockDim.x) {
    const int32_t i = perm[q];
    spos[q] = pos[i];
    smom[q] = mom[i];
  }
}

// Near-field correction, one warp per cell: up to kT of the cell's particles
// are the targets of a pass, held in shared memory (read as broadcasts).  The
// candidate sources of the neighbourhood are rows of cells trimmed to the
// cell-level distance bound of the near radius, each one contiguous range of
// the cell-ordered copies.  The rows are listed once per cell (start and
// prefix offset in shared memory) and their ranges are concatenated, so the
// lanes split one flat candidate index space: every sweep of the warp covers
// 32 candidates whatever the rows' lengths.  Each lane sweeps its candidates
// in increasing order, and every target's sum is finished by a fixed shuffle
// tree, so results are deterministic.
template <bool kForce>
__global__ void __launch_bounds__(128) k_correction_cells(const CellGrid* __restrict__ grids, int n_scenes,
                                                          int64_t n_cells, const int32_t* __restrict__ perm,
                                                          const int32_t* __restrict__ start,
                                                          const float4* __restrict__ spos,
                                                          const float4* __restrict__ smom, float4* __restrict__ corr,
                                                          const int32_t* __restrict__ skip_scene,
                                                          const double* __restrict__ done_flags, int done_stride,
                                                          const int32_t* __restrict__ done_count, int done_total) {
  constexpr int kT = 8;
  constexpr int kRows = 81;  // (2R + 1)^2 row slots, R <= 4 (cells are at least h wide)
  if (done_count && *done_count >= done_total) return;
  __shared__ float s_tbl[40];
  __shared__ float4 s_tp[4][kT], s_tm[4][kT];
  __shared__ int32_t s_rb[4][kRows], s_ro[4][kRows + 1];
  if (threadIdx.x < 40) s_tbl[threadIdx.x] = c_fit_tbl[threadIdx.x];
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int wi = threadIdx.x >> 5;
  const int64_t n_warps = int64_t(gridDim.x) * (blockDim.x >> 5);
  for (int64_t c = int64_t(blockIdx.x) * (blockDim.x >> 5) + wi; c < n_cells; c += n_warps) {
    const int32_t cb = start[c], ce = start[c + 1];
    if (cb == ce) continue;
    int lo = 0, hi = n_scenes - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (grids[mid].cell_off <= c) lo = mid;
      else hi = mid - 1;
    }
    if (done_flags && done_flags[int64_t(lo) * done_stride] != 0.0) continue;  // scene's solve stopped
    if (skip_scene && skip_scene[lo]) continue;  // scene evaluated by the exact-branch kernels
    const CellGrid& g = grids[lo];
    const int64_t lc = c - g.cell_off;
    const int ix = int(lc % g.nx), iy = int((lc / g.nx) % g.ny), iz = int(lc / (int64_t(g.nx) * g.ny));
    const int R = kForce ? g.reach_force : g.reach_field;
    const float near2 = kForce ? g.pc.near2_force : g.pc.near2_field;
    const float cs = 1.f / g.inv_cs;
    const float inv_h = g.pc.inv_h, ih3 = g.pc.ih3, ih4k = g.pc.ih4_over_k;
    float cA, cB;
    if (kForce) clamped_force_coeffs(near2, cA, cB);
    else clamped_field_coeffs(near2, cA, cB);
    // Row list of this cell: slot i = (dy, dz) in row-major order; a row
    // outside the grid or beyond the near radius has length 0.
    const int side = 2 * R + 1, n_slots = side * side;
    int32_t total = 0;
    __syncwarp();
    for (int i0 = 0; i0 < n_slots; i0 += 32) {
      const int i = i0 + lane;
      int32_t sb = 0, len = 0;
      if (i < n_slots) {
        const int dy = i % side - R, dz = i / side - R;
        const int cy = iy + dy, cz = iz + dz;
        const float gy = float(max(abs(dy) - 1, 0)) * cs, gz = float(max(abs(dz) - 1, 0)) * cs;
        const float rem = near2 - gz * gz - gy * gy;
        if (cy >= 0 && cy < g.ny && cz >= 0 && cz < g.nz && rem >= 0.f) {
          const int dxm = min(R, int(sqrtf(rem) * g.inv_cs) + 1);
          const int cx0 = max(ix - dxm, 0), cx1 = min(ix + dxm, g.nx - 1);
          const int64_t row = g.cell_off + (int64_t(cz) * g.ny + cy) * g.nx;
          sb = start[row + cx0];
          len = start[row + cx1 + 1] - sb;
        }
      }
      int32_t inc = len;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int32_t v = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += v;
      }
      if (i < n_slots) {
        s_rb[wi][i] = sb;
        s_ro[wi][i] = total + inc - len;
      }
      total += __shfl_sync(0xffffffffu, inc, 31);
    }
    if (lane == 0) s_ro[wi][n_slots] = total;
    __syncwarp();
    for (int32_t t0 = cb; t0 < ce; t0 += kT) {
      const int nt = min(kT, ce - t0);
      __syncwarp();
      if (lane < nt) {
        s_tp[wi][lane] = spos[t0 + lane];
        if (kForce) s_tm[wi][lane] = smom[t0 + lane];
      }
      __syncwarp();
      float acc[kT][3];
#pragma unroll
      for (int t = 0; t < kT; ++t) acc[t][0] = acc[t][1] = acc[t][2] = 0.f;
      {
        int r = 0;  // this lane's row cursor (its candidates only increase)
        for (int32_t k = lane; k < total; k += 32) {
          while (s_ro[wi][r + 1] <= k) ++r;
          const int32_t q = s_rb[wi][r] + (k - s_ro[wi][r]);
          {
            const float4 pj = spos[q];
            const float4 mj = smom[q];
#pragma unroll
            for (int t = 0; t < kT; ++t) {
              if (t < nt) {
                const float4 tp = s_tp[wi][t];
                const float dx = tp.x - pj.x, dy2 = tp.y - pj.y, dz2 = tp.z - pj.z;
                const float r2 = dx * dx + dy2 * dy2 + dz2 * dz2;
                if (kForce ? (r2 <= near2) : (r2 < near2)) {
                  if (kForce) {
                    const float4 tm = s_tm[wi][t];
                    float P, Q;
                    force_near_coeffs_fast(r2, s_tbl, inv_h, ih4k, P, Q);
                    const float dP = P - cA, dQ = Q - cB;
                    const float ds = dx * mj.x + dy2 * mj.y + dz2 * mj.z;
                    const float dm = dx * tm.x + dy2 * tm.y + dz2 * tm.z;
                    const float sm = mj.x * tm.x + mj.y * tm.y + mj.z * tm.z;
                    const float u = dP * ds, v = dP * dm, wv = dP * sm + dQ * ds * dm;
                    acc[t][0] += dx * wv + tm.x * u + mj.x * v;
                    acc[t][1] += dy2 * wv + tm.y * u + mj.y * v;
                    acc[t][2] += dz2 * wv + tm.z * u + mj.z * v;
                  } else {
                    float al, be;
                    field_near_coeffs_fast(r2, inv_h, ih3, al, be);
                    const float t3 = 3.f * (dx * mj.x + dy2 * mj.y + dz2 * mj.z) * (al - cA);
                    const float db = be - cB;
                    acc[t][0] += dx * t3 - mj.x * db;
                    acc[t][1] += dy2 * t3 - mj.y * db;
                    acc[t][2] += dz2 * t3 - mj.z * db;
                  }
                }
              }
            }
          }
        }
      }
      const float scale = kForce ? float(kForceK) : float(kInv4Pi);
#pragma unroll
      for (int t = 0; t < kT; ++t) {
        if (t < nt) {
#pragma unroll
          for (int k = 0; k < 3; ++k) {
            float v = acc[t][k];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            acc[t][k] = v;
          }
          if (lane == 0) corr[perm[t0 + t]] = make_float4(acc[t][0] * scale, acc[t][1] * scale, acc[t][2] * scale, 0.f);
        }
      }
    }
  }
}

// Targets are either the binned particles themselves (tpos == nullptr; they
// are visited in cell order so a warp's neighbours share cells) or a separate
// set tpos[0..n_total) of targets of scene 0.
template <bool kForce>
__global__ void __launch_bounds__(128) k_correction(const CellGrid* __restrict__ grids, int n_scenes,
                                                    int64_t n_total, const int32_t* __restrict__ perm,
                                                    const int32_t* __restrict__ start,
                                                    const float4* __restrict__ pos, const float4* __restrict__ mom,
                                                    const float4* __restrict__ tpos,
                                                    float4* __restrict__ corr) {
  for (int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; k < n_total;
       k += int64_t(gridDim.x) * blockDim.x) {
    const int64_t i = tpos ? k : int64_t(perm[k]);
    const CellGrid& g = grids[tpos ? 0 : scene_of(grids, n_scenes, i)];
    const float4 pi = tpos ? tpos[i] : pos[i];
    const float4 mi = tpos ? make_float4(0.f, 0.f, 0.f, 0.f) : mom[i];
    int ix, iy, iz;
    cell_coords(g, pi.x, pi.y, pi.z, ix, iy, iz);
    const int R = kForce ? g.reach_force : g.reach_field;
    const float near2 = kForce ? g.pc.near2_force : g.pc.near2_field;
    float cA, cB;  // clamped far coefficients of the packed loop
    if (kForce) clamped_force_coeffs(near2, cA, cB);
    else clamped_field_coeffs(near2, cA, cB);
    float s1[3] = {0.f, 0.f, 0.f}, s2[3] = {0.f, 0.f, 0.f};
    for (int dz = -R; dz <= R; ++dz) {
      const int cz = iz + dz;
      if (cz < 0 || cz >= g.nz) continue;
      for (int dy = -R; dy <= R; ++dy) {
        const int cy = iy + dy;
        if (cy < 0 || cy >= g.ny) continue;
        const int cx0 = max(ix - R, 0), cx1 = min(ix + R, g.nx - 1);
        const int64_t row = g.cell_off + (int64_t(cz) * g.ny + cy) * g.nx;
        // cells cx0..cx1 of a row are contiguous in the sorted list
        const int32_t b = start[row + cx0], e = start[row + cx1 + 1];
        for (int32_t q = b; q < e; ++q) {
          const int32_t j = perm[q];
          const float4 pj = pos[j];
          const float dx = pi.x - pj.x, dy2 = pi.y - pj.y, dz2 = pi.z - pj.z;
          const float r2 = dx * dx + dy2 * dy2 + dz2 * dz2;
          if (kForce ? (r2 <= near2) : (r2 < near2)) {
            const float4 mj = mom[j];
            if (kForce)
              force_near_correction(dx, dy2, dz2, mj.x, mj.y, mj.z, mi.x, mi.y, mi.z, g.pc, cA, cB, s1);
            else
              field_near_correction(dx, dy2, dz2, mj.x, mj.y, mj.z, g.pc, cA, cB, s1, s2);
          }
        }
      }
    }
    float4 o;
    if (kForce) {
      const float c = float(kForceK);
      o = make_float4(s1[0] * c, s1[1] * c, s1[2] * c, 0.f);
    } else {
      const float c = float(kInv4Pi);
      o = make_float4((3.f * s1[0] - s2[0]) * c, (3.f * s1[1] - s2[1]) * c, (3.f * s1[2] - s2[2]) * c, 0.f);
    }
    corr[i] = o;
  }
}

// Tensor correction at separate targets (single-scene list): corr[2i] =
// (xx, yy, zz, 0), corr[2i + 1] = (xy, xz, yz, 0) of the exact minus the
// clamped force tensor over the sources within 4h, in the output units.
__global__ void __launch_bounds__(128) k_tensor_correction(const CellGrid* __restrict__ grids, int64_t nt,
                                                           const int32_t* __restrict__ perm,
                                                           const int32_t* __restrict__ start,
                                                           const float4* __restrict__ pos,
                                                           const float4* __restrict__ mom,
                                                           const float4* __restrict__ tpos,
                                                           float4* __restrict__ corr) {
  const CellGrid& g = grids[0];
  const int R = g.reach_force;
  const float near2 = g.pc.near2_force;
  float cA, cB;
  clamped_force_coeffs(near2, cA, cB);
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < nt; i += int64_t(gridDim.x) * blockDim.x) {
    const float4 pi = tpos[i];
    int ix, iy, iz;
    cell_coords(g, pi.x, pi.y, pi.z, ix, iy, iz);
    float t[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    for (int dz = -R; dz <= R; ++dz) {
      const int cz = iz + dz;
      if (cz < 0 || cz >= g.nz) continue;
      for (int dy = -R; dy <= R; ++dy) {
        const int cy = iy + dy;
        if (cy < 0 || cy >= g.ny) continue;
        const int cx0 = max(ix - R, 0), cx1 = min(ix + R, g.nx - 1);
        const int64_t row = g.cell_off + (int64_t(cz) * g.ny + cy) * g.nx;
        const int32_t b = start[row + cx0], e = start[row + cx1 + 1];
        for (int32_t q = b; q < e; ++q) {
          const int32_t j = perm[q];
          const float4 pj = pos[j];
          const float dx = pi.x - pj.x, dy2 = pi.y - pj.y, dz2 = pi.z - pj.z;
          if (dx * dx + dy2 * dy2 + dz2 * dz2 <= near2) {
            const float4 mj = mom[j];
            tensor_near_correction(dx, dy2, dz2, mj.x, mj.y, mj.z, g.pc, cA, cB, t);
          }
        }
      }
    }
    const float c = float(kForceK);
    corr[2 * i] = make_float4(t[0] * c, t[1] * c, t[2] * c, 0.f);
    corr[2 * i + 1] = make_float4(t[3] * c, t[4] * c, t[5] * c, 0.f);
  }
}

__global__ void k_to_pairs(const float4* __restrict__ src, float4* __restrict__ dst, int64_t n,
                           const int32_t* __restrict__ done_count, int done_total) {
  if (done_count && *done_count >= done_total) return;
  const int64_t np = (n + 1) / 2;
  for (int64_t p = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; p < np; p += int64_t(gridDim.x) * blockDim.x) {
    const float4 a = src[2 * p];
    const float4 b = (2 * p + 1 < n) ? src[2 * p + 1] : make_float4(0.f, 0.f, 0.f, 0.f);
    dst[2 * p] = make_float4(a.x, b.x, a.y, b.y);
    dst[2 * p + 1] = make_float4(a.z, b.z, 0.f, 0.f);
  }
}

unsigned grid_for(int64_t n, int per_block = 256) {
  int64_t g = (n + per_block - 1) / per_block;
  if (g > 8192) g = 8192;
  return unsigned(g < 1 ? 1 : g);
}

}  // namespace

void to_pairs(const float4* src, float4* dst, int64_t n, cudaStream_t st, const int32_t* done_count,
              int done_total) {
  k_to_pairs<<<grid_for((n + 1) / 2), 256, 0, st>>>(src, dst, n, done_count, done_total);
}

mf_status CellList::build(const float4* pos4, const std::vector<CellSceneSpec>& scenes, cudaStream_t st,
                          double margin_h) {
  const int ns = int(scenes.size());
  if (ns == 0) return fail(MF_ERR_INVALID_ARG, "cell list: no scenes");
  n_scenes_ = ns;
  std::vector<int64_t> ranges(2 * size_t(ns));
  int64_t max_n = 0;
  n_total_ = 0;
  for (int s = 0; s < ns; ++s) {
    ranges[2 * s] = scenes[s].p_off;
    ranges[2 * s + 1] = scenes[s].n;
    max_n = std::max(max_n, scenes[s].n);
    n_total_ += scenes[s].n;
  }
  if (n_total_ >= (int64_t(1) << 31)) return fail(MF_ERR_INVALID_ARG, "cell list: too many particles");
  MF_TRY(bbox_.reserve(sizeof(int32_t) * 6 * ns + ranges.size() * sizeof(int64_t) + 64));
  int32_t* bbox = bbox_.as<int32_t>();
  int64_t* d_ranges = reinterpret_cast<int64_t*>(bbox_.as<char>() + ((sizeof(int32_t) * 6 * ns + 63) / 64) * 64);
  MF_CUDA_TRY(cudaMemcpyAsync(d_ranges, ranges.data(), ranges.size() * sizeof(int64_t), cudaMemcpyHostToDevice, st));
  k_bbox_init<<<grid_for(6 * ns), 256, 0, st>>>(bbox, ns);
  const unsigned gx = std::min<unsigned>(grid_for(max_n), 256);
  k_bbox<<<dim3(gx, unsigned(ns)), 256, 0, st>>>(pos4, d_ranges, bbox);
  MF_CUDA_TRY(cudaGetLastError());
  std::vector<int32_t> hb(6 * size_t(ns));
  MF_CUDA_TRY(cudaMemcpyAsync(hb.data(), bbox, hb.size() * sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  MF_CUDA_TRY(cudaStreamSynchronize(st));

  host_grids_.assign(size_t(ns), CellGrid{});
  host_bbox_.assign(6 * size_t(ns), 0.0);
  for (size_t k = 0; k < hb.size(); ++k) host_bbox_[k] = double(ord2f(hb[k]));
  int64_t cells = 0, prefix = 0;
  for (int s = 0; s < ns; ++s) {
    CellGrid& g = host_grids_[size_t(s)];
    const double h = scenes[s].h;
    double lo[3], ext[3];
    for (int c = 0; c < 3; ++c) {
      lo[c] = ord2f(hb[6 * s + c]) - margin_h * h;
      ext[c] = std::max(0.0, double(ord2f(hb[6 * s + 3 + c])) + margin_h * h - lo[c]);
      if (!std::isfinite(lo[c]) || !std::isfinite(ext[c])) return fail(MF_ERR_INVALID_ARG, "non-finite positions");
    }
    // Cells a hair wider than h (about 8 particles at h = 2 spacings): a point
    // closer than 2h (4h) to a target then always lies within 2 (4) cells of
    // it, whatever the rounding of the cell map.
    double cs = h * (1.0 + 1e-4);
    // Keep the grid at most ~8 cells per particle: widen cells for sparse scenes.
    const double cap = std::max(64.0, 8.0 * double(scenes[s].n));
    for (int it = 0; it < 64; ++it) {
      const double c3 = (std::floor(ext[0] / cs) + 1) * (std::floor(ext[1] / cs) + 1) * (std::floor(ext[2] / cs) + 1);
      if (c3 <= cap) break;
      cs *= 1.25;
    }
    g.ox = float(lo[0]);
    g.oy = float(lo[1]);
    g.oz = float(lo[2]);
    g.inv_cs = float(1.0 / cs);
    g.nx = int32_t(std::floor(ext[0] / cs)) + 1;
    g.ny = int32_t(std::floor(ext[1] / cs)) + 1;
    g.nz = int32_t(std::floor(ext[2] / cs)) + 1;
    g.reach_field = int32_t(std::ceil(2.0 * h / cs));
    g.reach_force = int32_t(std::ceil(4.0 * h / cs));
    g.cell_off = cells;
    g.p_off = scenes[s].p_off;
    g.n = scenes[s].n;
    g.k_off = prefix;
    g.pc = make_pair_consts<float>(h);
    cells += int64_t(g.nx) * g.ny * g.nz;
    prefix += scenes[s].n;
  }
  n_cells_ = cells;
  MF_TRY(grids_.reserve(sizeof(CellGrid) * size_t(ns)));
  MF_CUDA_TRY(cudaMemcpyAsync(grids_.ptr, host_grids_.data(), sizeof(CellGrid) * size_t(ns), cudaMemcpyHostToDevice,
                              st));
  MF_TRY(cell_start_.reserve_slack(sizeof(int32_t) * size_t(cells + 1)));
  MF_TRY(cursor_.reserve_slack(sizeof(int32_t) * size_t(cells + 1)));
  MF_TRY(scan_tiles_.reserve_slack(sizeof(int32_t) * size_t((cells + kScanTile - 1) / kScanTile + 1)));
  MF_TRY(perm_.reserve(sizeof(int32_t) * size_t(n_total_)));
  MF_TRY(perm_tmp_.reserve(sizeof(int32_t) * size_t(n_total_)));
  MF_TRY(cell_of_.reserve(sizeof(int32_t) * size_t(n_total_)));
  MF_TRY(spos_.reserve(sizeof(float4) * size_t(n_total_)));
  MF_TRY(smom_.reserve(sizeof(float4) * size_t(n_total_)));
  return rebin(pos4, st);
}

mf_status CellList::rebin(const float4* pos4, cudaStream_t st) {
  const int64_t cells = n_cells_;
  const int ns = n_scenes_;
  int32_t* counts = cursor_.as<int32_t>();
  MF_CUDA_TRY(cudaMemsetAsync(counts, 0, sizeof(int32_t) * size_t(cells + 1), st));
  const CellGrid* dg = grids_.as<CellGrid>();
  k_count<<<grid_for(n_total_), 256, 0, st>>>(pos4, dg, ns, n_total_, counts, cell_of_.as<int32_t>());
  {
    const int64_t tiles = (cells + kScanTile - 1) / kScanTile;
    int32_t* tsum = scan_tiles_.as<int32_t>();
    if (tiles > 0) k_scan_tiles<<<unsigned(tiles), kScanThreads, 0, st>>>(counts, cells, tsum);
    k_scan_tile_sums<<<1, kScanThreads, 0, st>>>(tsum, tiles, cell_start_.as<int32_t>(), cells);
    if (tiles > 0) k_scan_apply<<<unsigned(tiles), kScanThreads, 0, st>>>(counts, cells, tsum, cell_start_.as<int32_t>());
  }
  MF_CUDA_TRY(cudaMemcpyAsync(cursor_.ptr, cell_start_.ptr, sizeof(int32_t) * size_t(cells), cudaMemcpyDeviceToDevice,
                              st));
  k_scatter<<<grid_for(n_total_), 256, 0, st>>>(dg, ns, n_total_, cell_of_.as<int32_t>(), cursor_.as<int32_t>(),
                                                perm_tmp_.as<int32_t>());
  k_sort_cells<<<grid_for(cells * 32), 256, 0, st>>>(cell_start_.as<int32_t>(), cells, perm_tmp_.as<int32_t>(),
                                                     perm_.as<int32_t>());
  MF_CUDA_TRY(cudaGetLastError());
  return MF_OK;
}

static unsigned cell_grid(int64_t cells) {
  int64_t g = cells;
  if (g > 65535) g = 65535;
  return unsigned(g < 1 ? 1 : g);
}

mf_status CellList::field_correction(const float4* pos4, const float4* mom4, float4* corr, cudaStream_t st,
                                     const double* done_flags, int done_stride, const int32_t* done_count,
                                     int done_total) const {
  k_gather_sorted<<<grid_for(n_total_), 256, 0, st>>>(perm_.as<int32_t>(), pos4, mom4, n_total_, spos_.as<float4>(),
                                                      smom_.as<float4>(), done_count, done_total);
  k_correction_cells<false><<<cell_grid((n_cells_ + 3) / 4), 128, 0, st>>>(
      grids_.as<CellGrid>(), n_scenes_, n_cells_, perm_.as<int32_t>(), cell_start_.as<int32_t>(), spos_.as<float4>(),
      smom_.as<float4>(), corr, skip_field_on_ ? skip_field_.as<int32_t>() : nullptr, done_flags, done_stride, done_count, done_total);
  MF_CUDA_TRY(cudaGetLastError());
  return MF_OK;
}

mf_status CellList::field_correction_at(const float4* tpos4, int64_t nt, const float4* pos4, const float4* mom4,
                                        float4* corr, cudaStream_t st) const {
  if (n_scenes_ != 1) return fail(MF_ERR_INVALID_ARG, "separate targets need a single-scene cell list");
  k_correction<false><<<grid_for(nt, 128), 128, 0, st>>>(grids_.as<CellGrid>(), n_scenes_, nt,
                                                          perm_.as<int32_t>(), cell_start_.as<int32_t>(), pos4, mom4,
                                                          tpos4, corr);
  MF_CUDA_TRY(cudaGetLastError());
  return MF_OK;
}

mf_status CellList::tensor_correction_at(const float4* tpos4, int64_t nt, const float4* pos4, const float4* mom4,
                                         float4* corr2, cudaStream_t st) const {
  if (n_scenes_ != 1) return fail(MF_ERR_INVALID_ARG, "separate targets need a single-scene cell list");
  k_tensor_correction<<<grid_for(nt, 128), 128, 0, st>>>(grids_.as<CellGrid>(), nt, perm_.as<int32_t>(),
                                                         cell_start_.as<int32_t>(), pos4, mom4, tpos4, corr2);
  MF_CUDA_TRY(cudaGetLastError());
  return MF_OK;
}

mf_status CellList::set_skips(const std::vector<int32_t>& field, const std::vector<int32_t>& force) {
  // A list without skips is not passed to the kernels; its buffer is kept
  // (freeing would wait for every stream of the device).
  auto put = [&](const std::vector<int32_t>& v, DevBuf& b, bool& on) -> mf_status {
    bool any = false;
    for (int32_t x : v) any = any || x != 0;
    on = any;
    if (!any) return MF_OK;
    if (int(v.size()) != n_scenes_) return fail(MF_ERR_INVALID_ARG, "skip list size");
    MF_TRY(b.reserve(v.size() * sizeof(int32_t)));
    MF_CUDA_TRY(cudaMemcpy(b.ptr, v.data(), v.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
    return MF_OK;
  };
  MF_TRY(put(field, skip_field_, skip_field_on_));
  MF_TRY(put(force, skip_force_, skip_force_on_));
  return MF_OK;
}

mf_status CellList::force_correction(const float4* pos4, const float4* mom4, float4* corr, cudaStream_t st) const {
  k_gather_sorted<<<grid_for(n_total_), 256, 0, st>>>(perm_.as<int32_t>(), pos4, mom4, n_total_, spos_.as<float4>(),
                                                      smom_.as<float4>(), nullptr, 0);
  k_correction_cells<true><<<cell_grid((n_cells_ + 3) / 4), 128, 0, st>>>(
      grids_.as<CellGrid>(), n_scenes_, n_cells_, perm_.as<int32_t>(), cell_start_.as<int32_t>(), spos_.as<float4>(),
      smom_.as<float4>(), corr, skip_force_on_ ? skip_force_.as<int32_t>() : nullptr, nullptr, 0, nullptr, 0);
  MF_CUDA_TRY(cudaGetLastError());
  return MF_OK;
}

}  // namespace mfgb
