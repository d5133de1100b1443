// step_device.cuh -- the device side shared by the single-run kernels
// (kernels.cu) and the ensemble kernels (kernels_ens.cu): the transforms,
// the bodies of the four step kernels, the small device helpers and the
// launch-size helpers.  Two translation units compile in parallel.
#pragma once
// The four kernels of one qgw time step on GB300 (sm_103a), for the plain
// FP64 path (T = double) and the compensated FP32 path (T = float, q held
// as hi + lo).
//
// One reference step (timestep, src/timestep.h:114-167) is
//   K1 rows   : apply the pending AB3 update of the previous step, project
//               layers onto vertical modes, forward DST-I along x
//   K2 columns: forward DST-I along y, Helmholtz divide, inverse DST-I
//               along y                                  (invert_pv core)
//   K3 rows   : inverse DST-I along x, back-project modes onto layers -> psi
//   K4 tiles  : RHS (Arakawa Jacobian, beta, viscosity, hyperviscosity,
//               wind, bottom drag, topography) -> f0, CFL maximum; the last
//               block advances dt/t and computes the AB3 coefficients
// The AB3 update q += c0 f0 + c1 f1 + c2 f2 needs the CFL-limited dt of the
// same step, i.e. a reduction over all of psi, so it is applied by the next
// step's K1 (or by the flush kernel at the end of a call), which saves one
// full pass over q, f0, f1, f2.
//
// Shared-memory rows use the padded layout of dst_core.h (pr/pc); work
// loops map item -> (row, index) by a shift and a mask when the item count
// per row is a power of two (block_items), by one division otherwise.
#include <cuda_runtime.h>

#include <algorithm>

#include "dst_blue.h"
#include "dst_fixed.cuh"
#include "periodic.cuh"
#include "kernels.h"
#include "qgw_device.cuh"

namespace qgw {

constexpr int NT = 256;          // threads per block in every step kernel
constexpr int GMAX = 16;         // max rows of one batched DST in a block
// The projection coefficients of a row kernel's mode (layer) group,
// cst[l * GMAX + g], sit at the start of its dynamic shared memory, before
// the work buffers: nl * GMAX values, rounded to whole 16-byte vectors.
template <typename T> __host__ __device__ inline size_t cst_bytes(int nl) {
  return ((size_t)nl * GMAX * sizeof(T) + 15) / 16 * 16;
}
constexpr int TX = 32, TYD = 16;  // RHS tile (interior points): width, default height (16 or 32)
constexpr double TEPS = 1e-9;    // src/timestep.h:16
constexpr double HUGEV = 1e30;   // src/qg.c:43

// columns per K2 tile: 32-byte rows of FP32 (8) and FP64 (4) values by
// default, 16-byte rows (half as many columns) as the alternative, and one
// column per tile for the chirp-z columns whose two buffers per column leave
// no room for more
template <typename T> struct ColsPer { static constexpr int value = 32 / (int)sizeof(T); };
template <typename T> __host__ __device__ inline int col_width(const StepArgs<T>& a) {
  return (a.CT == ColsPer<T>::value / 2 || a.CT == 1) ? a.CT : ColsPer<T>::value;
}

// --------------------------------------------------------------- DST block
// Batched DST-I of nrows rows (row r at A + r*ld, padded input format) by
// the whole block; B is the second work buffer.  Returns the buffer that
// holds the output.
template <typename T>
__device__ __forceinline__ T* dst_block_generic(T* A, T* B, int nrows, int ld, const DstGeom& g,
                                                const DstTables<T>& tb, T* tot) {
  const int tid = threadIdx.x + threadIdx.y * blockDim.x, nth = blockDim.x * blockDim.y;
  const int H = g.H;
  block_items(nrows, H, [&](int r, int i) { dst_pre_item<T>(A + r * ld, B + r * ld, i + 1, g, tb.pre); });
  __syncthreads();
  T* src = B;
  T* dst = A;
  int Ns = 1;
  for (int p = 0; p < g.npass; ++p) {
    const int R = g.radix[p];
    stockham_pass_block<T>(R, src, dst, nrows, ld, Ns, H, tb.tw);
    __syncthreads();
    Ns *= R;
    T* t = src; src = dst; dst = t;
  }
  // split: items k = 0..H/2 per row
  block_items(nrows, H / 2 + 1,
              [&](int r, int k) { dst_split_item<T>((const C2<T>*)(src + r * ld), dst + r * ld, k, g, tb.spl); });
  __syncthreads();
  const int nc = g.nchunk;
  block_items(nrows, nc, [&](int r, int c) { tot[r * 32 + c] = dst_scan_chunk<T>(dst + r * ld, c, g); });
  __syncthreads();
  const int warp = tid >> 5, lane = tid & 31, nwarp = nth >> 5;
  for (int r = warp; r < nrows; r += nwarp) {
    T incl = lane < nc ? tot[r * 32 + lane] : T(0);
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const T u = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += u;
    }
    T ex = __shfl_up_sync(0xffffffffu, incl, 1);
    if (lane == 0) ex = T(0);
    __syncwarp();
    if (lane < nc) tot[r * 32 + lane] = ex;
  }
  __syncthreads();
  block_items(nrows, nc, [&](int r, int c) {
    if (c > 0) dst_scan_fix<T>(dst + r * ld, c, tot[r * 32 + c], g);
  });
  __syncthreads();
  return dst;
}

// Chirp-z DST-I (dst_blue.h) of nrows rows in A (x_j at index j), B the
// second buffer, both of row_len = L complex values: chirp, L-point FFT,
// multiply by the chirp's transform (conjugated), FFT, output Y_k at index
// k; returns the buffer that holds the output.  g.H = L, g's radices are
// L's, tb.tw holds L's twiddles.
template <typename T>
__device__ __forceinline__ T* dst_block_blue(T* A, T* B, int nrows, int ld, const DstGeom& g, const DstTables<T>& tb) {
  const int M = g.M, L = g.H;
  block_items(nrows, L, [&](int r, int m) { blue_chirp_item<T>(A + r * ld, (C2<T>*)(B + r * ld), m, M, tb.bc); });
  __syncthreads();
  T* O = cfft_block<T>(B, A, nrows, ld, g, tb.tw, nullptr);
  block_items(nrows, L, [&](int r, int k) { blue_mul_item<T>((C2<T>*)(O + r * ld), k, tb.bz); });
  __syncthreads();
  T* D = cfft_block<T>(O, O == A ? B : A, nrows, ld, g, tb.tw, nullptr);
  T* out = D == A ? B : A;
  const T invL = T(1) / T(L);  // a power of two: exact
  block_items(nrows, M, [&](int r, int k) { blue_out_item<T>((const C2<T>*)(D + r * ld), out + r * ld, k, invL, tb.bc); });
  __syncthreads();
  return out;
}

// Block DST of any supported length: the power-of-two lengths M = 128..2048
// use the compile-time specialisations of dst_fixed.cuh (FP32 M = 512 and
// 1024: one warp per row, in place, the result in A), others (mixed radix
// 2, 3, 5, 7) the generic loops.
// HL != 0: a kernel specialised for half-length HL (its launcher checked the
// run's length), whose code then holds that transform alone -- the step
// kernels of the common lengths keep their instruction stream small; HL = -1:
// the chirp-z form (the lengths the half-length FFT cannot take).
template <typename T, int HL = 0>
__device__ __forceinline__ T* dst_block(T* A, T* B, int nrows, int ld, const DstGeom& g, const DstTables<T>& tb,
                                        T* tot) {
  if constexpr (HL == 512) {
    if constexpr (sizeof(T) == 4) return dst_block_warp_f32<9>(A, nrows, ld, tb);
    else return dst_block_fixed<T, 9>(A, B, nrows, ld, tb);
  }
  if constexpr (HL == -1) return dst_block_blue<T>(A, B, nrows, ld, g, tb);
  switch (g.H) {
    case 64: return dst_block_fixed<T, 6>(A, B, nrows, ld, tb);
    case 128: return dst_block_fixed<T, 7>(A, B, nrows, ld, tb);
    case 256:
      if constexpr (sizeof(T) == 4) return dst_block_warp_f32<8>(A, nrows, ld, tb);
      else return dst_block_fixed<T, 8>(A, B, nrows, ld, tb);
    case 512:
      if constexpr (sizeof(T) == 4) return dst_block_warp_f32<9>(A, nrows, ld, tb);
      else return dst_block_fixed<T, 9>(A, B, nrows, ld, tb);
    case 1024: return dst_block_fixed<T, 10>(A, B, nrows, ld, tb);
    default: return dst_block_generic<T>(A, B, nrows, ld, g, tb, tot);
  }
}

__device__ __forceinline__ void slabs(int si, int& s0, int& s1, int& s2) {
  const int m = si % 3;
  s0 = (3 - m) % 3;
  s1 = (4 - m) % 3;
  s2 = (5 - m) % 3;
}

// The AB3 update q + c0 f0 + c1 f1 + c2 f2 (src/timestep.h:138), with the
// FMAs written out so that every kernel that applies it rounds the same way.
template <typename T>
__device__ __forceinline__ T ab3_plain(T q, T c0, T c1, T c2, T f0, T f1, T f2) {
  return fmaT(c2, f2, fmaT(c1, f1, fmaT(c0, f0, q)));
}
__device__ __forceinline__ float ab3_increment(float c0, float c1, float c2, float f0, float f1, float f2) {
  return fmaT(c2, f2, fmaT(c1, f1, c0 * f0));
}

// Compensated add of an increment d to (hi, lo).
__device__ __forceinline__ void comp_add(float& hi, float& lo, float d) {
  const float s = hi + d;
  const float bp = s - hi;
  const float err = (hi - (s - bp)) + (d - bp);
  const float l2 = lo + err;
  const float h2 = s + l2;
  lo = l2 - (h2 - s);
  hi = h2;
}

// a run constant in the arithmetic type: the double itself, or its FP32 copy
// made on the host (no conversion on the device)
template <typename T> __device__ __forceinline__ T pick(double d, float f);
template <> __device__ __forceinline__ double pick<double>(double d, float) { return d; }
template <> __device__ __forceinline__ float pick<float>(double, float f) { return f; }

// Asynchronous global -> shared element copies (no register staging), so the
// independent tile loads of a block are all in flight at once.
template <typename T>
__device__ __forceinline__ void cp_async_elem(T* smem_dst, const T* gsrc) {
  const unsigned int d = (unsigned int)__cvta_generic_to_shared(smem_dst);
  if constexpr (sizeof(T) == 8)
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(gsrc) : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// Start bringing a transform's tables into L1 (the s_j table, the pass
// twiddles, the split's cos/sin: ~8 KiB at M = 1024, read by every thread
// at each transform), one 128-byte line per thread, without waiting.
__device__ __forceinline__ void prefetch_l1(const void* p) {
  asm volatile("prefetch.global.L1 [%0];\n" ::"l"(p));
}
template <typename T>
__device__ __forceinline__ void prefetch_tables_l1(const DstTables<T>& t, int M) {
  const int tid = threadIdx.x + threadIdx.y * blockDim.x, nth = blockDim.x * blockDim.y;
  const int H = M / 2;
  const char* base[3] = {(const char*)t.sj, (const char*)t.twp, (const char*)t.spl};
  const int bytes[3] = {(H + 1) * (int)sizeof(T), H * (int)sizeof(C2<T>), (H / 2 + 1) * (int)sizeof(C2<T>)};
#pragma unroll
  for (int r = 0; r < 3; ++r)
    if (base[r])
      for (int off = tid * 128; off < bytes[r]; off += nth * 128) prefetch_l1(base[r] + off);
}

// Tensor-memory-accelerator tile loads completing on a shared-memory
// mbarrier (one elected thread issues them; every thread waits, bounded).
__device__ __forceinline__ unsigned int smem_u32(const void* p) { return (unsigned int)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(unsigned long long* bar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(bar)) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, unsigned int bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned int parity) {
  unsigned int ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// bounded wait: false when the limit ran out (the caller records an error)
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long* bar, unsigned int parity,
                                                  int limit = kWaitIters) {
  for (int it = 0; it < limit; ++it)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int x, int y, int z,
                                            unsigned long long* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];\n" ::
          "r"(smem_u32(dst)),
      "l"(map), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}
// order this thread's earlier generic shared-memory accesses before later
// asynchronous-proxy (TMA) writes to the same memory
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
}

// Records and weights of the 4-D forcing at time t (calc_4d_forcing,
// src/forcing.h:259-287): q_forc = w1 rec[i1] + w2 rec[i2].
struct Forc4D {
  int i1, i2;
  double w1, w2;
};
__device__ __forceinline__ Forc4D forc4d_at(double t, double dt_forc, int nrec) {
  Forc4D r;
  const double fl = floor(t / dt_forc);
  r.i1 = ((int)fl) % nrec;
  r.i2 = (r.i1 + 1) % nrec;
  r.w2 = t / dt_forc - (int)fl;
  r.w1 = 1 - r.w2;
  return r;
}
// q + q_forc * dt for one point (the reference's order: the weighted sum,
// then the product with dt, then the add)
template <typename T>
__device__ __forceinline__ T forc4d_term(const T* rec1, const T* rec2, size_t o, T w1, T w2, T dt) {
  return (w1 * rec1[o] + w2 * rec2[o]) * dt;
}

// ------------------------------------------------------- mode projections
// The nl x G coefficients of one mode group are staged in shared memory as
// cst[l * GMAX + gg] (zero for gg >= G), so one vector load serves a row of
// the group and the group loops have a compile-time width GB >= G.  A padded
// slot multiplies a zero value by a zero coefficient, which leaves every
// accumulator unchanged.
template <int GB, typename T>
__device__ __forceinline__ void ld_coefs(const T* __restrict__ c, T* r) {
  if constexpr (sizeof(T) == 4 && GB >= 4) {
#pragma unroll
    for (int v = 0; v < GB / 4; ++v) {
      const float4 x = reinterpret_cast<const float4*>(c)[v];
      r[4 * v] = x.x; r[4 * v + 1] = x.y; r[4 * v + 2] = x.z; r[4 * v + 3] = x.w;
    }
  } else if constexpr (sizeof(T) == 8 && GB >= 2) {
#pragma unroll
    for (int v = 0; v < GB / 2; ++v) {
      const double2 x = reinterpret_cast<const double2*>(c)[v];
      r[2 * v] = x.x; r[2 * v + 1] = x.y;
    }
  } else {
#pragma unroll
    for (int g = 0; g < GB; ++g) r[g] = c[g];
  }
}

// smallest compile-time group width that holds G rows
__device__ __forceinline__ int group_width(int G) { return G <= 1 ? 1 : G <= 2 ? 2 : G <= 4 ? 4 : G <= 8 ? 8 : 16; }

// ------------------------------------------------------------------ K1
// One block per row j.  Mode groups are processed in turn by the same block:
// the AB3 update is applied (and q written) while forming the first group,
// and later groups re-read the updated q written by the same thread, so no
// block ever reads a q value another block may be updating.  Each thread
// accumulates the G modes of its points in registers, layer by layer.
// frow (optional): the stochastic forcing of row j, added to layer 0 as
// frow * sqdt after the AB3 update (src/timestep.h:143-150)
// FK: 0 no forcing, 1 stochastic forcing only (layer 0), 2 either or both
// -- separate instantiations, so that each loop carries only the forcing it
// applies; 3: no update pending, q comes from the caller's array a.qin
// (reference layout) and is stored into the run's field on the way.
// Point i of the row goes to index i + xo of its mode row (xo = 1: the DST's
// x_{i+1} at index i+1; xo = 0: the real FFT's x_i at index i).
template <typename T, bool COMP, int GB, int FK>
__device__ __forceinline__ void project_fwd(const StepArgs<T>& a, int j, bool upd, T c0, T c1, T c2, const T* f0,
                                            const T* f1, const T* f2, int G, T* A, int ld, const T* cst,
                                            const T* frow, T sqdt, const T* r1, const T* r2, T w1, T w2,
                                            T dtf, int xo) {
  if constexpr (FK == 3) {
    // q from the caller's host array: four layers' loads in flight per
    // point (the link's latency is several microseconds), then the stores
    // into the run's field and the projection
    const size_t hs = (size_t)(a.ny + 2) * (a.nx + 2);
    for (int i = threadIdx.x; i < a.nx; i += NT) {
      T acc[GB];
#pragma unroll
      for (int g = 0; g < GB; ++g) acc[g] = T(0);
      const double* __restrict__ src = a.qin + (size_t)(j + 1) * (a.nx + 2) + (i + 1);
      const size_t o0 = (size_t)j * a.pitch + i;
      for (int l0 = 0; l0 < a.nl; l0 += 4) {
        double x[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) x[u] = l0 + u < a.nl ? src[(size_t)(l0 + u) * hs] : 0.0;
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int l = l0 + u;
          if (l >= a.nl) break;
          const size_t o = o0 + (size_t)l * a.lstride;
          T v;
          if constexpr (COMP) {
            const float hi = (float)x[u];
            a.q[o] = (T)hi;
            a.qlo[o] = (T)(float)(x[u] - (double)hi);
            v = (T)hi;
          } else {
            v = (T)x[u];
            a.q[o] = v;
          }
          T c[GB];
          ld_coefs<GB, T>(cst + l * GMAX, c);
#pragma unroll
          for (int g = 0; g < GB; ++g) acc[g] = fmaT(c[g], v, acc[g]);
        }
      }
      const int pi = pr<T>(i + xo);
#pragma unroll
      for (int g = 0; g < GB; ++g)
        if (g < G) A[g * ld + pi] = acc[g];
    }
  } else {
  // FP32: two points per pass (i and i + NT, the second absent past the
  // row's end), every layer's loads of both issued before either is used:
  // the fields stream from HBM/L2 and one point's chain of layers alone
  // leaves the loads' latency exposed.  FP64 (bound by its FP64 pipe, and
  // without registers for a second point's 16-wide groups): one point.
  constexpr int PP = sizeof(T) == 4 ? 2 : 1;
  T* __restrict__ qh = a.q;
  T* __restrict__ ql = a.qlo;
  const T* __restrict__ g0 = f0;
  const T* __restrict__ g1 = f1;
  const T* __restrict__ g2 = f2;
  // one layer of one point: the pending AB3 update (and forcing) of q,
  // stored back, and the value the projection takes
  auto layer = [&](int i, size_t o, int l, T qv, T lov, T a0, T a1, T a2) -> T {
    if (COMP) {
      float hi = (float)qv;
      if (upd) {
        float lo = (float)lov;
        const float d = ab3_increment((float)c0, (float)c1, (float)c2, (float)a0, (float)a1, (float)a2);
        comp_add(hi, lo, d);
        if (FK == 1 && l == 0) comp_add(hi, lo, (float)frow[i] * (float)sqdt);
        if (FK == 2) {
          if (frow && l == 0) comp_add(hi, lo, (float)frow[i] * (float)sqdt);
          if (r1) comp_add(hi, lo, (float)forc4d_term<T>(r1, r2, o, w1, w2, dtf));
        }
        qh[o] = (T)hi;
        ql[o] = (T)lo;
      }
      return (T)hi;
    } else {
      T v = qv;
      if (upd) {
        v = ab3_plain<T>(v, c0, c1, c2, a0, a1, a2);
        if (FK == 1 && l == 0) v = v + frow[i] * sqdt;
        if (FK == 2) {
          if (frow && l == 0) v = v + frow[i] * sqdt;
          v = v + forc4d_term<T>(r1, r2, o, w1, w2, dtf);
        }
        qh[o] = v;
      }
      return v;
    }
  };
  for (int i = threadIdx.x; i < a.nx; i += PP * NT) {
    const int i2 = i + NT;
    const bool two = PP == 2 && i2 < a.nx;
    T acc[GB], acc2[GB];
#pragma unroll
    for (int g = 0; g < GB; ++g) acc[g] = acc2[g] = T(0);
    size_t o = (size_t)j * a.pitch + i;
    for (int l = 0; l < a.nl; ++l, o += a.lstride) {
      const size_t o2 = o + NT;
      const T x = qh[o], x2 = two ? qh[o2] : T(0);
      T lo = T(0), lo2 = T(0), a0 = T(0), a1 = T(0), a2 = T(0), b0 = T(0), b1 = T(0), b2 = T(0);
      if (upd) {
        if (COMP) { lo = ql[o]; if (two) lo2 = ql[o2]; }
        a0 = g0[o]; a1 = g1[o]; a2 = g2[o];
        if (two) { b0 = g0[o2]; b1 = g1[o2]; b2 = g2[o2]; }
      }
      const T v = layer(i, o, l, x, lo, a0, a1, a2);
      const T v2 = two ? layer(i2, o2, l, x2, lo2, b0, b1, b2) : T(0);
      T c[GB];
      ld_coefs<GB, T>(cst + l * GMAX, c);
#pragma unroll
      for (int g = 0; g < GB; ++g) {
        acc[g] = fmaT(c[g], v, acc[g]);
        acc2[g] = fmaT(c[g], v2, acc2[g]);
      }
    }
    const int pi = pr<T>(i + xo);
#pragma unroll
    for (int g = 0; g < GB; ++g)
      if (g < G) A[g * ld + pi] = acc[g];
    if (two) {
      const int pi2 = pr<T>(i2 + xo);
#pragma unroll
      for (int g = 0; g < GB; ++g)
        if (g < G) A[g * ld + pi2] = acc2[g];
    }
  }
  }
}

// PER: doubly periodic basin -- real FFT of the row instead of the DST-I;
// the spectral row holds X_0..X_H as (re, im) pairs (nx + 2 reals).
template <typename T, bool COMP, bool PER, int HL = 0>
__device__ __forceinline__ void body_rows_fwd(const StepArgs<T>& a, int step_mode, int j, unsigned char* smem_raw,
                                              T* tot, T* cst) {
  DevState* st = a.state;
  if (step_mode && !st->active) return;
  const int ld = row_len<T>(a.gx);
  T* A = (T*)smem_raw;
  T* B = A + (size_t)a.G1 * ld;
  const bool ab3 = step_mode && st->pending;
  int s0 = 0, s1 = 0, s2 = 0;
  slabs(st->step_index, s0, s1, s2);
  const T c0 = (T)st->c0, c1 = (T)st->c1, c2 = (T)st->c2;
  const size_t fs = (size_t)a.nl * a.lstride;
  const T* f0 = a.fab + s0 * fs;
  const T* f1 = a.fab + s1 * fs;
  const T* f2 = a.fab + s2 * fs;
  const int tid = threadIdx.x;
  // FP32 groups of 9..12 modes run at width 12 (three 16-byte coefficient
  // vectors), the common 10-layer case without six idle accumulators
  const int GB = (sizeof(T) == 4 && a.G1 > 8 && a.G1 <= 12) ? 12 : group_width(a.G1);
  if (!PER) prefetch_tables_l1(a.tx, a.gx.M);
  const T* frow = (ab3 && a.fr.on) ? a.fr.field + (size_t)j * a.pitch : nullptr;
  const T sqdt = frow ? (T)sqrt(st->dt) : T(0);
  const T* r1 = nullptr;
  const T* r2 = nullptr;
  T w1 = T(0), w2 = T(0), dtf = T(0);
  if (ab3 && a.nrec > 0) {
    const Forc4D fw = forc4d_at(st->t_prev, a.dt_forc, a.nrec);
    const size_t rs = (size_t)a.nl * a.lstride;
    r1 = a.frec + fw.i1 * rs;
    r2 = a.frec + fw.i2 * rs;
    w1 = (T)fw.w1;
    w2 = (T)fw.w2;
    dtf = (T)st->dt;
  }
  // ceil(nl / G1) groups of balanced sizes (at most G1 each)
  const int ng = (a.nl + a.G1 - 1) / a.G1, gq = a.nl / ng, gr = a.nl - gq * ng;
  for (int gi = 0, m0 = 0; gi < ng; m0 += gq + (gi < gr), ++gi) {
    const int G = gq + (gi < gr);
    const bool upd = ab3 && m0 == 0;
    for (int w = tid; w < a.nl * GMAX; w += NT) {
      const int l = w / GMAX, g = w - l * GMAX;
      cst[w] = g < G ? a.cl2m[(size_t)(m0 + g) * a.nl + l] : T(0);
    }
    __syncthreads();
    const int fk = (a.qin && m0 == 0) ? 3 : !upd ? 0 : r1 ? 2 : frow ? 1 : 0;
#define QGW_PF(GBV, F) project_fwd<T, COMP, GBV, F>(a, j, upd, c0, c1, c2, f0, f1, f2, G, A, ld, cst, frow, sqdt, r1, \
                                                  r2, w1, w2, dtf, PER ? 0 : 1)
#define QGW_PF_GB(F)                 \
  switch (GB) {                      \
    case 1: QGW_PF(1, F); break;     \
    case 2: QGW_PF(2, F); break;     \
    case 4: QGW_PF(4, F); break;     \
    case 8: QGW_PF(8, F); break;     \
    case 12:                         \
      if constexpr (sizeof(T) == 4) {\
        QGW_PF(12, F);               \
        break;                       \
      }                              \
      [[fallthrough]];               \
    default: QGW_PF(16, F); break;   \
  }
    // the compensated path has registers for one forced loop only
    if (fk == 3) {
      QGW_PF_GB(3)
    } else if (fk == 2 || (COMP && fk == 1)) {
      QGW_PF_GB(2)
    } else if (fk == 1) {
      if constexpr (!COMP) QGW_PF_GB(1)
    } else {
      QGW_PF_GB(0)
    }
#undef QGW_PF_GB
#undef QGW_PF
    __syncthreads();
    T* O = PER ? rfft_block<T>(A, B, G, ld, a.gx, a.tx) : dst_block<T, HL>(A, B, G, ld, a.gx, a.tx, tot);
    // spectral row: the real FFT's X_0..X_H as (re, im) pairs from index 0,
    // or the DST's Y_1..Y_{M-1} from index 1
    const int nout = PER ? a.nx + 2 : a.nx, yo = PER ? 0 : 1;
    for (int gg = 0; gg < G; ++gg) {
      T* dstrow = a.spec + (size_t)(m0 + gg) * a.lstride + (size_t)j * a.pitch;
      for (int i = threadIdx.x; i < nout; i += NT) dstrow[i] = O[gg * ld + pr<T>(i + yo)];
    }
    __syncthreads();
  }
}

// ------------------------------------------------------------------ K2
// CT columns of one mode per block (CT * sizeof(T) = 32 bytes: two 16-byte
// vectors per row, one thread per row), transposed into shared memory so
// that each column is a contiguous padded row.
template <typename T, int CT>
__device__ __forceinline__ void load_cols(const T* __restrict__ src, T* v) {
  constexpr int NV = CT * (int)sizeof(T) / 16, PV = 16 / (int)sizeof(T);
  static_assert(NV >= 1 && CT * sizeof(T) == 16 * NV, "whole 16-byte vectors");
  const uint4* p = reinterpret_cast<const uint4*>(src);
#pragma unroll
  for (int n = 0; n < NV; ++n) {
    const uint4 u = p[n];
    const T* a = reinterpret_cast<const T*>(&u);
#pragma unroll
    for (int c = 0; c < PV; ++c) v[n * PV + c] = a[c];
  }
}
// load_cols with streaming (evict-first) loads: data read once
template <typename T, int CT>
__device__ __forceinline__ void load_cols_stream(const T* __restrict__ src, T* v) {
  constexpr int NV = CT * (int)sizeof(T) / 16, PV = 16 / (int)sizeof(T);
  static_assert(NV >= 1 && CT * sizeof(T) == 16 * NV, "whole 16-byte vectors");
  const uint4* p = reinterpret_cast<const uint4*>(src);
#pragma unroll
  for (int n = 0; n < NV; ++n) {
    const uint4 u = __ldcs(p + n);
    const T* a = reinterpret_cast<const T*>(&u);
#pragma unroll
    for (int c = 0; c < PV; ++c) v[n * PV + c] = a[c];
  }
}
template <typename T, int CT>
__device__ __forceinline__ void store_cols(T* __restrict__ dst, const T* v) {
  constexpr int NV = CT * (int)sizeof(T) / 16, PV = 16 / (int)sizeof(T);
  uint4* p = reinterpret_cast<uint4*>(dst);
#pragma unroll
  for (int n = 0; n < NV; ++n) {
    uint4 u;
    T* a = reinterpret_cast<T*>(&u);
#pragma unroll
    for (int c = 0; c < PV; ++c) a[c] = v[n * PV + c];
    p[n] = u;
  }
}

template <typename T, bool COMP, int CT, int HL = 0>
__device__ __forceinline__ void body_cols(const StepArgs<T>& a, int step_mode, int bx, int m, unsigned char* smem_raw,
                                          T* tot) {
  DevState* st = a.state;
  if (step_mode && !st->active) return;
  const int k0 = bx * CT;
  const int CTb = min(CT, a.nx - k0);
  const int ld = row_len<T>(a.gy);
  const bool zm = COMP && a.zeta_mode;
  // Two pairs of CT-row buffers, [A | C] and [B | D]: the forward DST runs on
  // A with B as work buffer; the divide overwrites its output O with psi_hat
  // and, in zeta mode, writes the second field into the CT rows after O; the
  // inverse DST then transforms both at once (2 CT rows) with the other pair
  // as work buffer.  Column jj + 1 of a tile row holds point jj (x_{jj+1}).
  T* A = (T*)smem_raw;
  T* B = A + (size_t)(zm ? 2 : 1) * CT * ld;
  T* S = a.spec + (size_t)m * a.lstride;
  const int ny = a.ny;
  prefetch_tables_l1(a.ty, a.gy.M);
  // 16-byte vectors need 16-byte aligned rows (vec_cols); the last tile then
  // reads the padding column (index nx < pitch), never past the row.  RB
  // rows per pass, all their loads in flight before any store (two 32-byte
  // rows); streaming loads (the tile is read once), which leave L1 to the
  // tables.
  constexpr int RB = 2;
  // Thread t takes the points jj = t - 1 + u NT (tile index jj + 1 = t +
  // u NT), so that each warp's shared-memory accesses cover whole 128-byte
  // pad periods (one wavefront per access).
  // (a one-column tile, narrower than a vector, reads element by element)
  constexpr bool VEC = CT * sizeof(T) % 16 == 0;
  const bool vec = VEC && a.vec_cols != 0;
  for (int j0 = threadIdx.x - 1; j0 < ny; j0 += RB * NT) {
    T vv[RB][CT];
#pragma unroll
    for (int u = 0; u < RB; ++u) {
      const int jj = j0 + u * NT;
      if (jj >= 0 && jj < ny) {
        const T* src = S + (size_t)jj * a.pitch + k0;
        if constexpr (VEC) {
          if (vec) {
            load_cols_stream<T, CT>(src, vv[u]);
            continue;
          }
        }
        for (int c = 0; c < CT; ++c) vv[u][c] = c < CTb ? src[c] : T(0);
      }
    }
#pragma unroll
    for (int u = 0; u < RB; ++u) {
      const int jj = j0 + u * NT;
      if (jj >= 0 && jj < ny) {
        const int pj = pr<T>(jj + 1);
#pragma unroll
        for (int c = 0; c < CT; ++c) A[c * ld + pj] = vv[u][c];
      }
    }
  }
  __syncthreads();
  T* O = dst_block<T, HL>(A, B, CT, ld, a.gy, a.ty, tot);
  T* C = O + (size_t)CT * ld;  // the second field's rows (zeta mode)
  const double iRd2 = a.iRd2[m];
  // power of the 5-point symbol in the second field: L psi (zeta mode 1) or
  // the whole hyperviscosity chain L^nsweep psi (zeta mode 2)
  const int zpow = (COMP && a.zeta_mode == 2) ? a.nsweep : 1;
  const float ird2f = COMP ? a.iRd2f[m] : 0.f;
  const float normf = a.fc[FC_NORM], lx2f = a.fc[FC_LX2], ly2f = a.fc[FC_LY2];
  // the tile's per-column table values, the same for every row
  float lsqc[CT], sxc[CT];
#pragma unroll
  for (int c = 0; c < CT; ++c) {
    const int k = min(k0 + c, a.nx - 1);
    lsqc[c] = COMP ? a.Lsqf[k] : 0.f;
    sxc[c] = zm ? a.sx2f[k] : 0.f;
  }
  // RB rows per pass, their per-row loads issued before any is used
  for (int j0 = threadIdx.x - 1; j0 < ny; j0 += RB * NT) {
    T h4[RB][CT];
    float ksq4[RB], sy4[RB];
#pragma unroll
    for (int u = 0; u < RB; ++u) {
      const int jj = j0 + u * NT;
      if (jj < 0 || jj >= ny) continue;
      if (!COMP) {
        const T* hrow = (const T*)(a.hinv + (size_t)m * a.lstride + (size_t)jj * a.pitch + k0);
        if constexpr (VEC) {
          if (vec) {
            load_cols<T, CT>(hrow, h4[u]);
            continue;
          }
        }
        for (int c = 0; c < CT; ++c) h4[u][c] = c < CTb ? hrow[c] : T(0);
      } else {
        ksq4[u] = a.Ksqf[jj];
        sy4[u] = zm ? a.sy2f[jj] : 0.f;
      }
    }
#pragma unroll
    for (int u = 0; u < RB; ++u) {
      const int jj = j0 + u * NT;
      if (jj < 0 || jj >= ny) continue;
      const int pj = pr<T>(jj + 1);
      if (!COMP) {
#pragma unroll
        for (int c = 0; c < CT; ++c) O[c * ld + pj] *= h4[u][c];
      } else {
#pragma unroll
        for (int c = 0; c < CT; ++c) {
          const int k = min(k0 + c, a.nx - 1);
          float x;
          if (m == 0 && jj < a.low_k64 && k < a.low_k64) {
            // barotropic mode, lowest wavenumbers: divide in FP64
            const double fact = -(a.Lsq[k] + a.Ksq[jj] + iRd2);
            x = (float)((double)O[c * ld + pj] / fact / a.norm);
          } else {
            const float fact = -((lsqc[c] + ksq4[u]) + ird2f);
            x = (float)O[c * ld + pj] / (fact * normf);
          }
          O[c * ld + pj] = (T)x;
          if (zm) {
            // spectral discrete Laplacian of psi: lambda(k, j) * psi_hat with
            // lambda = -4/Delta^2 (sin^2 kx + sin^2 ky), the exact symbol of
            // the 5-point Laplacian with zero ghosts in the DST basis; applied
            // zpow times, one factor after the other (no underflow of
            // lambda^zpow at the lowest wavenumbers)
            const float lam = lx2f * sxc[c] + ly2f * sy4[u];
            float z = lam * x;
            for (int s = 1; s < zpow; ++s) z = z * lam;
            C[c * ld + pj] = (T)z;
          }
        }
      }
    }
  }
  __syncthreads();
  T* Oth = (O == A) ? B : A;
  T* O2 = dst_block<T, HL>(O, Oth, zm ? 2 * CT : CT, ld, a.gy, a.ty, tot);
  T* S2 = zm ? a.spec2 + (size_t)m * a.lstride : nullptr;
  T v[CT];
  for (int jj = threadIdx.x - 1; jj < ny; jj += NT) {
    if (jj < 0) continue;
    const int pj = pr<T>(jj + 1);
#pragma unroll
    for (int c = 0; c < CT; ++c) v[c] = c < CTb ? O2[c * ld + pj] : T(0);
    T* dst = S + (size_t)jj * a.pitch + k0;
    if (vec) store_cols<T, CT>(dst, v);
    else
      for (int c = 0; c < CTb; ++c) dst[c] = v[c];
    if (zm) {
#pragma unroll
      for (int c = 0; c < CT; ++c) v[c] = c < CTb ? O2[(CT + c) * ld + pj] : T(0);
      T* dst2 = S2 + (size_t)jj * a.pitch + k0;
      if (vec) store_cols<T, CT>(dst2, v);
      else
        for (int c = 0; c < CTb; ++c) dst2[c] = v[c];
    }
  }
}

// ------------------------------------------------------------- K2 periodic
// Two complex columns k = 2 bx, 2 bx + 1 (one tile of four reals) of one mode
// per block: complex FFT along y, Helmholtz divide, backward FFT (as the
// conjugate of the forward FFT of the conjugate), in zeta mode also the
// spectral 5-point Laplacian of psi.  Columns k > nx/2 are padding.
template <typename T, bool COMP>
__device__ __forceinline__ void body_cols_per(const StepArgs<T>& a, int step_mode, int bx, int m, unsigned char* smem_raw) {
  constexpr int CC = 2;
  DevState* st = a.state;
  if (step_mode && !st->active) return;
  const int H = a.gx.H;  // x: complex columns k = 0..H
  const int k0 = bx * CC;
  const int ld = row_len<T>(a.gy);
  T* A = (T*)smem_raw;
  T* B = A + (size_t)CC * ld;
  T* C = B + (size_t)CC * ld;  // zeta mode only
  T* S = a.spec + (size_t)m * a.lstride;
  const int ny = a.ny;
  const int tid = threadIdx.x + threadIdx.y * blockDim.x;
  for (int jj = tid; jj < ny; jj += NT) {
    T v[4];
    load_cols<T, 4>(S + (size_t)jj * a.pitch + 2 * k0, v);
    const int pj = pc<T>(jj);
    C2<T>* A0 = (C2<T>*)A;
    C2<T>* A1 = (C2<T>*)(A + ld);
    C2<T> z0, z1;
    z0.x = v[0]; z0.y = v[1]; z1.x = v[2]; z1.y = v[3];
    A0[pj] = z0;
    A1[pj] = z1;
  }
  __syncthreads();
  T* O = cfft_block<T>(A, B, CC, ld, a.gy, a.ty.tw, a.ty.twp);
  const bool zm = COMP && a.zeta_mode;
  const int zpow = (COMP && a.zeta_mode == 2) ? a.nsweep : 1;  // as in body_cols
  const double iRd2 = a.iRd2[m];
  const float ird2f = COMP ? a.iRd2f[m] : 0.f;
  const float normf = a.fc[FC_NORM], lx2f = a.fc[FC_LX2], ly2f = a.fc[FC_LY2];
  for (int w = tid; w < CC * ny; w += NT) {
    const int c = w / ny, jj = w - c * ny;
    const int k = k0 + c;
    C2<T>* Oc = (C2<T>*)(O + c * ld);
    const int pj = pc<T>(jj);
    C2<T> X = Oc[pj];
    if (k > H || (k == 0 && jj == 0)) {
      // padding columns; the mean is removed (src/elliptic.h:115-118)
      X.x = T(0);
      X.y = T(0);
    } else if (!COMP) {
      const T h = (T)a.hinv[(size_t)m * a.lstride + (size_t)jj * a.pitch + k];
      X.x = X.x * h;
      X.y = X.y * h;
    } else {
      const int fy = jj <= ny / 2 ? jj : ny - jj;  // |y wavenumber index|
      if (m == 0 && fy < a.low_k64 && k < a.low_k64) {
        // barotropic mode, lowest wavenumbers: divide in FP64
        const double fact = -(a.Lsq[k] + a.Ksq[jj] + iRd2);
        X.x = (T)((double)X.x / fact / a.norm);
        X.y = (T)((double)X.y / fact / a.norm);
      } else {
        const float fact = -((a.Lsqf[k] + a.Ksqf[jj]) + ird2f);
        X.x = (T)((float)X.x / (fact * normf));
        X.y = (T)((float)X.y / (fact * normf));
      }
    }
    if (zm) {
      const int kk = k > H ? H : k;
      const float lam = lx2f * a.sx2f[kk] + ly2f * a.sy2f[jj];
      float zx = lam * (float)X.x, zy = lam * (float)X.y;
      for (int s = 1; s < zpow; ++s) {
        zx = zx * lam;
        zy = zy * lam;
      }
      C2<T> Z;
      Z.x = (T)zx;
      Z.y = -(T)zy;
      ((C2<T>*)(C + c * ld))[pj] = Z;
    }
    X.y = -X.y;  // conjugate: backward FFT = conj(FFT(conj))
    Oc[pj] = X;
  }
  __syncthreads();
  T* Oth = (O == A) ? B : A;
  T* O2 = cfft_block<T>(O, Oth, CC, ld, a.gy, a.ty.tw, a.ty.twp);
  for (int jj = tid; jj < ny; jj += NT) {
    const int pj = pc<T>(jj);
    const C2<T> z0 = ((const C2<T>*)O2)[pj];
    const C2<T> z1 = ((const C2<T>*)(O2 + ld))[pj];
    T v[4] = {z0.x, -z0.y, z1.x, -z1.y};
    store_cols<T, 4>(S + (size_t)jj * a.pitch + 2 * k0, v);
  }
  if (zm) {
    __syncthreads();
    T* O3 = cfft_block<T>(C, O2 == A ? B : A, CC, ld, a.gy, a.ty.tw, a.ty.twp);
    T* S2 = a.spec2 + (size_t)m * a.lstride;
    for (int jj = tid; jj < ny; jj += NT) {
      const int pj = pc<T>(jj);
      const C2<T> z0 = ((const C2<T>*)O3)[pj];
      const C2<T> z1 = ((const C2<T>*)(O3 + ld))[pj];
      T v[4] = {z0.x, -z0.y, z1.x, -z1.y};
      store_cols<T, 4>(S2 + (size_t)jj * a.pitch + 2 * k0, v);
    }
  }
}

// ------------------------------------------------------------------ K3
// One block per row j with its LAYER groups in turn, or (a grid of rows x
// groups, the FP64 default) one block per group of row j.  The mode -> layer
// projection is linear and acts point by point, so it commutes with the
// x-DST: each group first forms the spectral rows of its layers,
// sum_m cm2l[l][m] * spec_m (and of zeta from spec2 in zeta mode), then
// inverse-transforms them and writes psi_l (zeta_l) once.  The spectral rows
// of row j are re-read by each group (from cache); nothing is accumulated in
// global memory.  Column i goes to index i + xo of its row (xo = 1: the
// DST's input format).
template <typename T, bool ZM, int GB>
__device__ __forceinline__ void project_spec(const StepArgs<T>& a, int j, int G, T* A, int ld, const T* cst,
                                             int ncols, int xo) {
  // FP32: two columns per pass (i and i + NT), each mode's loads of both
  // issued before either is used (the spectral rows come from L2); FP64
  // (FP64-pipe bound, registers for one column's groups): one column
  constexpr int PP = sizeof(T) == 4 ? 2 : 1;
  const T* __restrict__ sp = a.spec;
  const T* __restrict__ sp2 = a.spec2;
  for (int i = threadIdx.x; i < ncols; i += PP * NT) {
    const bool two = PP == 2 && i + NT < ncols;
    T acc[GB], zacc[ZM ? GB : 1], acc2[GB], zacc2[ZM ? GB : 1];
#pragma unroll
    for (int g = 0; g < GB; ++g) {
      acc[g] = acc2[g] = T(0);
      if (ZM) zacc[g] = zacc2[g] = T(0);
    }
    size_t o = (size_t)j * a.pitch + i;
#pragma unroll 2
    for (int m = 0; m < a.nl; ++m, o += a.lstride) {
      const T v = sp[o], v2 = two ? sp[o + NT] : T(0);
      T z = T(0), z2 = T(0);
      if (ZM) {
        z = sp2[o];
        z2 = two ? sp2[o + NT] : T(0);
      }
      T c[GB];
      ld_coefs<GB, T>(cst + m * GMAX, c);
#pragma unroll
      for (int g = 0; g < GB; ++g) {
        acc[g] = fmaT(c[g], v, acc[g]);
        acc2[g] = fmaT(c[g], v2, acc2[g]);
        if (ZM) {
          zacc[g] = fmaT(c[g], z, zacc[g]);
          zacc2[g] = fmaT(c[g], z2, zacc2[g]);
        }
      }
    }
    const int pi = pr<T>(i + xo), pi2 = pr<T>(i + NT + xo);
#pragma unroll
    for (int g = 0; g < GB; ++g)
      if (g < G) {
        A[g * ld + pi] = acc[g];
        if (ZM) A[(G + g) * ld + pi] = zacc[g];
        if (two) {
          A[g * ld + pi2] = acc2[g];
          if (ZM) A[(G + g) * ld + pi2] = zacc2[g];
        }
      }
  }
}

// only >= 0: this block takes layer group `only` of row j alone (a K3 grid
// of rows x groups); only < 0: it takes every group of the row in turn
template <typename T, bool COMP, bool PER, int HL = 0>
__device__ __forceinline__ void body_rows_inv(const StepArgs<T>& a, int step_mode, int j, unsigned char* smem_raw,
                                              T* tot, T* cst, int only = -1) {
  DevState* st = a.state;
  if (step_mode && !st->active) return;
  const int ld = row_len<T>(a.gx);
  const bool zm = COMP && a.zeta_mode;
  const int Gb = a.G3;
  T* A = (T*)smem_raw;
  T* B = A + (size_t)(zm ? 2 * Gb : Gb) * ld;
  const int GB = group_width(Gb);
  if (!PER) prefetch_tables_l1(a.tx, a.gx.M);
  // ceil(nl / Gb) layer groups of balanced sizes (at most Gb each)
  const int ng = (a.nl + Gb - 1) / Gb, gq = a.nl / ng, gr = a.nl - gq * ng;
  const int g_begin = only < 0 ? 0 : only, g_end = only < 0 ? ng : min(only + 1, ng);
  for (int gi = g_begin, l0 = g_begin * gq + min(g_begin, gr); gi < g_end; l0 += gq + (gi < gr), ++gi) {
    const int G = gq + (gi < gr);
    for (int w = threadIdx.x; w < a.nl * GMAX; w += NT) {
      const int m = w / GMAX, g = w - m * GMAX;
      cst[w] = g < G ? a.cm2l[(size_t)(l0 + g) * a.nl + m] : T(0);
    }
    __syncthreads();
    const int ncols = PER ? a.nx + 2 : a.nx, xo = PER ? 0 : 1;
    if (zm) {
      switch (GB) {
        case 1: project_spec<T, true, 1>(a, j, G, A, ld, cst, ncols, xo); break;
        case 2: project_spec<T, true, 2>(a, j, G, A, ld, cst, ncols, xo); break;
        case 4: project_spec<T, true, 4>(a, j, G, A, ld, cst, ncols, xo); break;
        default: project_spec<T, true, 8>(a, j, G, A, ld, cst, ncols, xo); break;
      }
    } else {
      switch (GB) {
        case 1: project_spec<T, false, 1>(a, j, G, A, ld, cst, ncols, xo); break;
        case 2: project_spec<T, false, 2>(a, j, G, A, ld, cst, ncols, xo); break;
        case 4: project_spec<T, false, 4>(a, j, G, A, ld, cst, ncols, xo); break;
        case 8: project_spec<T, false, 8>(a, j, G, A, ld, cst, ncols, xo); break;
        default: project_spec<T, false, 16>(a, j, G, A, ld, cst, ncols, xo); break;
      }
    }
    __syncthreads();
    const int nrow = zm ? 2 * G : G;
    T* O = PER ? irfft_block<T>(A, B, nrow, ld, a.gx, a.tx) : dst_block<T, HL>(A, B, nrow, ld, a.gx, a.tx, tot);
    // periodic: x_{2m+1} is minus the imaginary part of the backward FFT
    // (x_i at index i); DST: x_{i+1} at index i + 1
    const T odd = PER ? T(-1) : T(1);
    for (int g = 0; g < G; ++g) {
      T* prow = a.psi + (size_t)(l0 + g) * a.lstride + (size_t)j * a.pitch;
      for (int i = threadIdx.x; i < a.nx; i += NT) {
        const T v = O[g * ld + pr<T>(i + xo)];
        prow[i] = (PER && (i & 1)) ? odd * v : v;
      }
      if (zm) {
        T* zrow = a.zeta + (size_t)(l0 + g) * a.lstride + (size_t)j * a.pitch;
        for (int i = threadIdx.x; i < a.nx; i += NT) {
          const T v = O[(G + g) * ld + pr<T>(i + xo)];
          zrow[i] = (PER && (i & 1)) ? odd * v : v;
        }
      }
    }
    __syncthreads();
  }
}

// ------------------------------------------------------------------ K4
__device__ __forceinline__ unsigned long long absbits(double v) {
  return (unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffULL;
}
// |v| as bits in the arithmetic width (non-negative floats order like their
// bit patterns); a float maximum is widened to double bits once per block
__device__ __forceinline__ unsigned long long absbits_native(double v) { return absbits(v); }
__device__ __forceinline__ unsigned int absbits_native(float v) { return __float_as_uint(v) & 0x7fffffffu; }
template <typename T> __device__ __forceinline__ unsigned long long widen_absbits(unsigned long long b) { return b; }
template <> __device__ __forceinline__ unsigned long long widen_absbits<float>(unsigned long long b) {
  // NaN and Inf stay above every finite value after widening
  return absbits((double)__uint_as_float((unsigned int)b));
}

// adjust_timestep's dt rule (src/timestep.h:69-111) and the AB3
// coefficients (src/timestep.h:130-133), by one thread.
static __device__ void scalar_update(DevState* st, double Delta, double cfl) {
  const unsigned long long bits = atomicMax(&st->maxbits, 0ULL);
  const bool bad = bits >= 0x7ff0000000000000ULL;
  double dt_max = HUGEV;
  const double maxabs = __longlong_as_double((long long)bits);
  if (!bad && maxabs != 0.0) {
    const double u = maxabs / Delta;
    const double dl = cfl * Delta / u;
    if (dl < dt_max) dt_max = dl;
  }
  const double t = st->t;
  double dt = st->dt;
  st->dt1 = st->dt0;
  st->dt0 = dt;
  if (dt < dt_max) dt = 2. * dt;
  if (dt > st->DT_max) dt = st->DT_max;
  if (dt > dt_max) dt = dt_max;
  const double t_out = st->t_out;
  if (t_out > t + TEPS) {
    const unsigned int n_step = (unsigned int)((t_out - t) / dt);
    if (n_step == 0)
      dt = t_out - t;
    else {
      const double d1 = (t_out - t) / n_step;
      if (d1 > dt * (1. + TEPS))
        dt = (t_out - t) / (n_step + 1);
      else if (d1 < dt)
        dt = d1;
    }
  }
  st->dt = dt;
  const double dt0 = st->dt0, dt1 = st->dt1;
  st->c0 = dt * (2 * dt * dt + 3 * dt * (2 * dt0 + dt1) + 6 * dt0 * (dt0 + dt1)) / (6 * dt0 * (dt0 + dt1));
  st->c1 = dt * dt * (-dt / 3 - dt0 / 2 - dt1 / 2) / (dt0 * dt1);
  st->c2 = dt * dt * (dt / 3 + dt0 / 2) / (dt1 * (dt0 + dt1));
  st->pending = 1;
  const double tn = t + dt;
  st->t_prev = t;
  st->t = tn;
  st->step_index += 1;
  st->steps_taken += 1;
  st->first = 0;
  if (bad) {
    st->active = 0; st->stop_reason = 3; st->nonfinite = 1;
  } else if (st->tend > 0 && !(tn < st->tend)) {
    st->active = 0; st->stop_reason = 2;
  } else if (fabs(tn - t_out) < TEPS * dt) {
    st->active = 0; st->stop_reason = 1;
  } else if (st->max_steps > 0 && st->steps_taken >= st->max_steps) {
    st->active = 0; st->stop_reason = 0;
  }
  st->maxbits = 0ULL;
  st->done_blocks = 0u;
}

// index g of a periodic dimension of n points brought into [0, n)
__device__ __forceinline__ int wrap_index(int g, int n) {
  const int r = g % n;
  return r < 0 ? r + n : r;
}

// Shared-memory layout of the RHS tile: psi-shaped arrays (psi, the two
// chain buffers) have HH = TY + 2R rows of TW = TX + 8 columns, tile column
// xx at TW offset TOX = 4 (xx = -4..TX+3, the span of one TMA box starting at
// the 16-byte aligned x = i0 - 4); the q tile has QH = TY + 2 rows of TW
// columns with the same column offset.  Each array starts 128-byte aligned.
constexpr int TW = TX + 8, TOX = 4;
template <typename T> __host__ __device__ constexpr int tile_round(int n) {
  return (n + (128 / (int)sizeof(T)) - 1) / (128 / (int)sizeof(T)) * (128 / (int)sizeof(T));
}

// Shared memory of the RHS kernels: NB input buffers (a TMA box set: psi
// with halo R, q with halo 1 and, in zeta mode 1, the raw zeta of the first
// sweep's region) followed by the work buffers (the chain's ping-pong and,
// for FP64, the centred differences).  Every array starts 128-byte aligned.
template <typename T, int R, int TY> struct RhsShape {
  static constexpr int HH = TY + 2 * R, QH = TY + 2, QW = TX + 2;
  static constexpr int TS = tile_round<T>(TW * HH), QS = tile_round<T>(TW * QH), ZS = tile_round<T>(TW * (HH - 2));
  static constexpr int IS = TS + QS + ZS;  // one input buffer
  static constexpr int DIFFS = sizeof(T) == 8 ? tile_round<T>(2 * QW * TY + 2 * TX * QH) : 0;
  static constexpr int WS = 2 * TS + DIFFS;  // work buffers
  static constexpr size_t bytes(int nb) { return sizeof(T) * ((size_t)nb * IS + WS) + 128; }
};
template <typename T> struct RhsIn {
  T* ps;  // HH x TW: psi with halo R
  T* qs;  // QH x TW: q with halo 1
  T* zt;  // (HH - 2) x TW: zeta over the first sweep's region (zeta mode 1)
};
template <typename T, int R, int TY> __device__ __forceinline__ RhsIn<T> rhs_in(unsigned char* base, int b) {
  using S = RhsShape<T, R, TY>;
  T* p = (T*)base + (size_t)b * S::IS;
  return RhsIn<T>{p, p + S::TS, p + S::TS + S::QS};
}
template <typename T, int R, int TY> __device__ __forceinline__ T* rhs_work(unsigned char* base, int nb) {
  return (T*)base + (size_t)nb * RhsShape<T, R, TY>::IS;
}

// Loads of one tile that do not go through TMA, into `in`: edge tiles
// (periodic: psi and q wrapped around; closed, where no tensor map exists:
// the three fields bounds-checked, zero outside the domain, as a TMA box
// reads them) and, where no tensor map exists, interior tiles by
// element-wise asynchronous copies (all three fields together).  A closed
// edge tile's ghost values of q (which need the whole psi tile) and of the
// chain are formed by rhs_tile_compute.  The caller synchronises the block
// afterwards.
template <typename T, bool COMP, int R, int TY, bool EDGE>
__device__ __forceinline__ void rhs_tile_fetch(const StepArgs<T>& a, int i0, int j0, int k, const RhsIn<T>& in) {
  constexpr int W = TW, HH = TY + 2 * R;
  constexpr int QW = TX + 2, QH = TY + 2;
  constexpr int XO = TOX;
  const int tid = threadIdx.x + threadIdx.y * 32;
  const int nx = a.nx, ny = a.ny, pitch = a.pitch;
  const T* psiL = a.psi + (size_t)k * a.lstride;
  const T* qL = a.q + (size_t)k * a.lstride;
  T* ps = in.ps;
  T* qs = in.qs;
  if (EDGE && a.periodic) {
    // periodic: every halo value is an interior value of the other side
    // (src/domain.h:225-256); tiles may be wider than the domain
    for (int w = tid; w < HH * (TX + 2 * R); w += NT) {
      const int y = w / (TX + 2 * R), xx = w - y * (TX + 2 * R) - R;
      ps[y * W + xx + XO] = psiL[(size_t)wrap_index(j0 + y - R, ny) * pitch + wrap_index(i0 + xx, nx)];
    }
    for (int w = tid; w < QH * QW; w += NT) {
      const int y = w / QW, xx = w - y * QW - 1;
      qs[y * W + xx + XO] = qL[(size_t)wrap_index(j0 + y - 1, ny) * pitch + wrap_index(i0 + xx, nx)];
    }
  } else if (EDGE) {
    // closed basin: what a TMA box with zero fill holds (the compute step
    // then writes the ghost values)
    for (int w = tid; w < HH * (TX + 2 * R); w += NT) {
      const int y = w / (TX + 2 * R), xx = w - y * (TX + 2 * R) - R;
      const int gi = i0 + xx, gj = j0 + y - R;
      T v = T(0);
      if (gi >= 0 && gi < nx && gj >= 0 && gj < ny) v = psiL[(size_t)gj * pitch + gi];
      ps[y * W + xx + XO] = v;
    }
    for (int w = tid; w < QH * QW; w += NT) {
      const int y = w / QW, xx = w - y * QW - 1;
      const int gi = i0 + xx, gj = j0 + y - 1;
      T v = T(0);
      if (gi >= 0 && gi < nx && gj >= 0 && gj < ny) v = qL[(size_t)gj * pitch + gi];
      qs[y * W + xx + XO] = v;
    }
    if (COMP && a.zeta_mode == 1 && a.nsweep >= 1) {
      constexpr int W1 = TX + 2 * R - 2, H1 = HH - 2;
      const T* zL = a.zeta + (size_t)k * a.lstride;
      for (int w = tid; w < W1 * H1; w += NT) {
        const int yr = w / W1, xr = w - yr * W1;
        const int gi = i0 + xr + 1 - R, gj = j0 + yr + 1 - R;
        T v = T(0);
        if (gi >= 0 && gi < nx && gj >= 0 && gj < ny) v = zL[(size_t)gj * pitch + gi];
        in.zt[yr * W + xr + 1 - R + XO] = v;
      }
    }
  } else {
    const T* src = psiL + (size_t)(j0 - R) * pitch + (i0 - R);
    for (int w = tid; w < HH * (TX + 2 * R); w += NT) {
      const int y = w / (TX + 2 * R), x = w - y * (TX + 2 * R);
      cp_async_elem(ps + y * W + x - R + XO, src + y * pitch + x);
    }
    const T* qsrc = qL + (size_t)(j0 - 1) * pitch + (i0 - 1);
    for (int w = tid; w < QH * QW; w += NT) {
      const int y = w / QW, x = w - y * QW;
      cp_async_elem(qs + y * W + x - 1 + XO, qsrc + y * pitch + x);
    }
    if (COMP && a.zeta_mode == 1 && a.nsweep >= 1) {
      constexpr int W1 = TX + 2 * R - 2, H1 = HH - 2;
      const T* zsrc = a.zeta + (size_t)k * a.lstride + (size_t)(j0 + 1 - R) * pitch + (i0 + 1 - R);
      for (int w = tid; w < W1 * H1; w += NT) {
        const int yr = w / W1, xr = w - yr * W1;
        cp_async_elem(in.zt + yr * W + xr + 1 - R + XO, zsrc + yr * pitch + xr);
      }
    }
    cp_async_wait_all();
  }
}

// An interior tile's boxes by TMA (one thread): psi (HH rows), q (QH rows)
// and, in zeta mode 1, zeta over the first sweep's region (HH - 2 rows), each
// TW columns from x = i0 - 4; the mbarrier `bar` collects the bytes.  The
// caller has synchronised the block since the buffers were last read.
template <typename T, bool COMP, int R, int TY>
__device__ __forceinline__ void rhs_tile_tma(const StepArgs<T>& a, int i0, int j0, int k, const RhsIn<T>& in,
                                             const CUtensorMap* tm, unsigned long long* bar) {
  constexpr int W = TW, HH = TY + 2 * R, QH = TY + 2;
  fence_proxy_async_smem();
  const bool z1 = COMP && a.zeta_mode == 1 && a.nsweep >= 1;
  const unsigned int bytes = (unsigned int)sizeof(T) * W * (HH + QH + (z1 ? HH - 2 : 0));
  mbar_expect_tx(bar, bytes);
  tma_load_3d(in.ps, &tm[0], i0 - TOX, j0 - R, k, bar);
  tma_load_3d(in.qs, &tm[1], i0 - TOX, j0 - 1, k, bar);
  if (z1) tma_load_3d(in.zt, &tm[2], i0 - TOX, j0 + 1 - R, k, bar);
}

// Block-uniform bounded wait for a tile's TMA bytes.  When the first wait
// (a.wait_iters polls) runs out, the run is flagged (QGW_ERR_TIMEOUT), the
// bytes get a second wait with the full limit (they may still land in this
// block's shared memory) and the tile is to be skipped: returns false.
template <typename T>
__device__ __forceinline__ bool rhs_tile_wait(const StepArgs<T>& a, unsigned long long* bar, unsigned int* phase) {
  const bool ok = __syncthreads_and(mbar_wait_bounded(bar, *phase, a.wait_iters)) != 0;
  if (!ok) {
    (void)mbar_wait_bounded(bar, *phase, kWaitIters);
    if (threadIdx.x == 0 && threadIdx.y == 0) a.state->dev_error = 1;
  }
  *phase ^= 1u;
  return ok;
}

// RHS tile of TX x TY points of one layer; block (32, 8); R = halo radius
// of psi (the number of hyperviscosity sweeps the tile runs, at least 1).
// EDGE: the tile plus its halo touches a wall, so ghost values follow
// adjust_bc (or wrap around, periodic); interior tiles (the vast majority)
// skip all of that.  The tile's inputs are in `in` and the block has been
// synchronised since they arrived; `wk` holds the work buffers.  Returns
// this thread's CFL maximum |dpsi| as bits in the arithmetic width.
// Z1: the run is in zeta mode 1 with R = nsweep sweeps (the compensated
// path's common case), which the compiler then knows: the sweep count, the
// chain's units and the buffers each sweep reads and writes.
template <typename T, bool COMP, int R, int TY, bool EDGE, bool Z1 = false>
__device__ __forceinline__ decltype(absbits_native(T(0))) rhs_tile_compute(const StepArgs<T>& a, int i0, int j0,
                                                                            int k, int step_index,
                                                                            const RhsIn<T>& in, T* wk) {
  constexpr int W = TW, HH = TY + 2 * R;
  constexpr int QW = TX + 2, QH = TY + 2;
  constexpr int XO = TOX;  // column of tile x = 0
  constexpr int TS = RhsShape<T, R, TY>::TS;
  T* ps = in.ps;              // HH x W, psi with halo R
  T* qs = in.qs;              // QH x W
  T* L0 = wk;                 // chain ping-pong
  T* L1 = L0 + TS;
  T* dyp = L1 + TS;           // TY x QW (FP64 only)
  T* dyq = dyp + QW * TY;
  T* dxp = dyq + QW * TY;     // QH x TX
  T* dxq = dxp + TX * QH;
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int nx = a.nx, ny = a.ny, pitch = a.pitch;
  const T* qL = a.q + (size_t)k * a.lstride;
  // zeta mode 1: the spectral L psi starts the chain and gives the drag;
  // zeta mode 2: the field is the whole chain L^nsweep psi (no sweeps here)
  const bool zm = Z1 || (COMP && a.zeta_mode == 1);
  const bool zm2 = !Z1 && COMP && a.zeta_mode == 2;
  const int ksweep = Z1 ? R : zm2 ? 0 : a.nsweep;  // Laplacian sweeps run on the tile
  const T* zetaL = (COMP && a.zeta_mode) ? a.zeta + (size_t)k * a.lstride : nullptr;
  // every double parameter converted once (conversions run on the FP64 pipe)
  const T d2 = pick<T>(a.Delta * a.Delta, a.fc[FC_D2]);
  const T cbc = pick<T>(a.cbc, a.fc[FC_CBC]);
  const T m_inv12 = pick<T>(-a.inv12d2, a.fc[FC_MINV12]), b2d = pick<T>(a.b2d, a.fc[FC_B2D]);
  const T nu_d2 = pick<T>(a.nu_d2, a.fc[FC_NUD2]), nuh = pick<T>(a.nuh_scaled, a.fc[FC_NUH]);
  const T nuhs = pick<T>(0.0, a.fc[FC_NUHS]), nuhd2 = pick<T>(0.0, a.fc[FC_NUHD2]);
  const T drag = pick<T>(a.drag_d2, a.fc[FC_DRAG]), topo_c = pick<T>(-(a.inv12d2 * a.topo_fac), a.fc[FC_TOPOC]);
#define PS(x, y) ps[((y) + R) * W + (x) + XO]
#define QS(x, y) qs[((y) + 1) * W + (x) + XO]
  const int tid = tx + ty * 32;
  const bool per = a.periodic != 0;
  // zeta mode 2: the chain value at this thread's points (x = tx, y = 16 b
  // + 2 ty + h; the FP32 Jacobian's mapping), loaded first so that its
  // latency overlaps the tile's shared-memory work
  static_assert(TY % 16 == 0, "tiles of 16-row bands");
  constexpr int NBAND = TY / 16;
  T hv[2 * NBAND];
#pragma unroll
  for (int h = 0; h < 2 * NBAND; ++h) hv[h] = T(0);
  if (zm2) {
#pragma unroll
    for (int h = 0; h < 2 * NBAND; ++h) {
      const int gi = i0 + tx, gj = j0 + 16 * (h >> 1) + 2 * ty + (h & 1);
      if (!EDGE || (gi < nx && gj < ny)) hv[h] = zetaL[(size_t)gj * pitch + gi];
    }
  }
  // q with one ghost point: adjust_bc(q, 1, psi), src/domain.h:308-348; the
  // interior values arrived with the tile (zero outside the domain)
  if (EDGE && !per) {
    for (int w = tid; w < QH * QW; w += NT) {
      const int y = w / QW, x = w - y * QW;
      const int xx = x - 1, yy = y - 1;
      const int gi = i0 + xx, gj = j0 + yy;
      const bool inx = gi >= 0 && gi < nx, iny = gj >= 0 && gj < ny;
      if (inx && iny) continue;
      T v = T(0);
      if (iny && gi == -1) v = cbc * PS(xx + 1, yy);
      else if (iny && gi == nx) v = cbc * PS(xx - 1, yy);
      else if (inx && gj == -1) v = cbc * PS(xx, yy + 1);
      else if (inx && gj == ny) v = cbc * PS(xx, yy - 1);
      qs[y * W + xx + XO] = v;
    }
  }
  // hyperviscosity chain (calc_diff, src/dynamics.h:13-44) on the tile with
  // a shrinking halo; sweeps are unscaled (no 1/Delta^2), the scale is in
  // nuh_scaled and in the ghost factors gh[s]; in zeta mode the first
  // sweep is the spectral zeta.  Unrolled over s so that every region
  // width is a compile-time constant.  Region of sweep s: tile rows
  // yy = s-R .. TY+R-s-1 (smem row yy + R), columns xx likewise (xx + XO).
  // Zeta mode 1 runs the chain on zeta = L psi / Delta^2 rather than L psi
  // (fold): an interior tile takes the zeta tile itself as the first
  // sweep's output, edge tiles divide their ghost values by Delta^2, and
  // the factor Delta^2 moves into the coefficient.  Every point's value is
  // then the same whatever tile holds it (the tile shape never changes the
  // result).
  const bool fold = zm && ksweep >= 1;
  const T* Lp = (fold && !EDGE) ? in.zt - W : ps;  // zt's row 0 is the first sweep's first row
  T* Lc = L0;
#pragma unroll
  for (int s = 1; s <= R; ++s) {
    if (s <= ksweep && !(s == 1 && fold && !EDGE)) {
      __syncthreads();
      const int Ws = TX + 2 * R - 2 * s, Hs = HH - 2 * s;
      const int cx = s - R + XO;  // smem column of the region's first point
      if (EDGE && per) {
        // periodic: no walls, the sweep is the Laplacian everywhere
        for (int w = tid; w < Ws * Hs; w += NT) {
          const int yr = w / Ws, xr = w - yr * Ws;
          const int o = (yr + s) * W + xr + cx;
          if (s == 1 && zm) {
            Lc[o] = zetaL[(size_t)wrap_index(j0 + yr + s - R, ny) * pitch + wrap_index(i0 + xr + s - R, nx)];
          } else {
            const T sum = (Lp[o + 1] + Lp[o - 1]) + (Lp[o + W] + Lp[o - W]);
            Lc[o] = fmaT(T(-4), Lp[o], sum);
          }
        }
      } else if (EDGE) {
        // ghost factor of sweep s (divided by Delta^2 in zeta mode 1)
        const T ghs = pick<T>(a.gh[s], a.fc[(fold ? FC_GHD1 : FC_GH1) + s - 1]);
        for (int w = tid; w < Ws * Hs; w += NT) {
          const int yr = w / Ws, xr = w - yr * Ws;
          const int xx = xr + s - R, yy = yr + s - R;
          const int gi = i0 + xx, gj = j0 + yy;
          const bool inx = gi >= 0 && gi < nx, iny = gj >= 0 && gj < ny;
          const int o = (yr + s) * W + xr + cx;
          T v = T(0);
          if (inx && iny) {
            if (s == 1 && zm) {
              v = in.zt[o - W];  // the zeta tile, one row up
            } else {
              const T sum = (Lp[o + 1] + Lp[o - 1]) + (Lp[o + W] + Lp[o - W]);
              v = fmaT(T(-4), Lp[o], sum);
            }
          } else if (iny && gi == -1) v = ghs * PS(xx + 1, yy);
          else if (iny && gi == nx) v = ghs * PS(xx - 1, yy);
          else if (inx && gj == -1) v = ghs * PS(xx, yy + 1);
          else if (inx && gj == ny) v = ghs * PS(xx, yy - 1);
          Lc[o] = v;
        }
      } else {
        // two vertically adjacent points per item (Hs is even), sharing
        // their column of four values; same arithmetic per point.  The
        // region's first 32 columns go one row pair per warp (each warp's
        // accesses in one row: no bank conflicts), its last Ws - 32 columns
        // (Ws >= 32) after them.
        auto pair = [&](int yp, int xr) {
          const int o = (2 * yp + s) * W + xr + cx;
          const T c0 = Lp[o - W], c1 = Lp[o], c2 = Lp[o + W], c3 = Lp[o + 2 * W];
          Lc[o] = fmaT(T(-4), c1, (Lp[o + 1] + Lp[o - 1]) + (c2 + c0));
          Lc[o + W] = fmaT(T(-4), c2, (Lp[o + W + 1] + Lp[o + W - 1]) + (c3 + c1));
        };
        static_assert(TX == 32, "one warp per row of the region's first 32 columns");
        for (int w = tid; w < 32 * (Hs / 2); w += NT) pair(w >> 5, w & 31);
        if (Ws > 32) {
          for (int w = tid; w < (Ws - 32) * (Hs / 2); w += NT) {
            const int yp = w / (Ws - 32);
            pair(yp, 32 + w - yp * (Ws - 32));
          }
        }
      }
      Lp = Lc;
      Lc = (Lc == L0) ? L1 : L0;
    }
  }
  __syncthreads();
  const size_t fs = (size_t)a.nl * a.lstride;
  int s0, s1, s2;
  slabs(step_index + 1, s0, s1, s2);
  T* fout = a.fab + s0 * fs + (size_t)k * a.lstride;
  const bool bottom = (k == a.nl - 1);
  decltype(absbits_native(T(0))) mymax_n = 0;
  const int x = tx;
  // the rest of the RHS at one point (src/dynamics.h:55-69) given its
  // Jacobian J and the centred differences dxp = psi_E - psi_W,
  // dyp = psi_N - psi_S (and, in zeta mode 2, the spectral chain value
  // hchain at the point); then the CFL maximum
  // (pc, pe, pn: psi at the point and its east and north neighbours)
  auto finish = [&](int y, T J, T dxp, T dyp, T hchain, T pc, T pe, T pn) {
    const int gi = i0 + x, gj = j0 + y;
    // rhs, src/dynamics.h:55-58: -J - beta psi_x + nu lap q + nu_h lap^n psi
    T f = fmaT(m_inv12, J, -(b2d * dxp));
    if (a.has_nu) {
      const T lq = fmaT(T(-4), QS(x, y), (QS(x + 1, y) + QS(x - 1, y)) + (QS(x, y + 1) + QS(x, y - 1)));
      f = fmaT(nu_d2, lq, f);
    }
    if (zm2) f = fmaT(nuhs, hchain, f);
    else if (a.nsweep > 0) f = fmaT(fold ? nuhd2 : nuh, Lp[(y + R) * W + x + XO], f);
    // surface wind (src/dynamics.h:66) and bottom drag + topography (:67-69)
    if (k == 0 && a.has_wind) f += a.wind[gj];
    if (bottom) {
      if (a.has_drag) {
        const T lp = zm ? d2 * zetaL[(size_t)gj * pitch + gi]
                        : fmaT(T(-4), PS(x, y), (PS(x + 1, y) + PS(x - 1, y)) + (PS(x, y + 1) + PS(x, y - 1)));
        f = fmaT(drag, lp, f);
      }
      if (a.has_topo) {
        // J(psi, topo) on the ghosted topography grid (reference layout)
        const int tp = nx + 2;
        const double* tb = a.topo + (size_t)(gj + 1) * tp + (gi + 1);
#define TP(dx, dy) ((T)tb[(dy) * tp + (dx)])
        const T jt = (dxp * (TP(0, 1) - TP(0, -1)) - dyp * (TP(1, 0) - TP(-1, 0))
                      + PS(x + 1, y) * (TP(1, 1) - TP(1, -1)) - PS(x - 1, y) * (TP(-1, 1) - TP(-1, -1))
                      - PS(x, y + 1) * (TP(1, 1) - TP(-1, 1)) + PS(x, y - 1) * (TP(1, -1) - TP(-1, -1))
                      + TP(0, 1) * (PS(x + 1, y + 1) - PS(x - 1, y + 1))
                      - TP(0, -1) * (PS(x + 1, y - 1) - PS(x - 1, y - 1))
                      - TP(1, 0) * (PS(x + 1, y + 1) - PS(x + 1, y - 1))
                      + TP(-1, 0) * (PS(x - 1, y + 1) - PS(x - 1, y - 1)));
#undef TP
        f = fmaT(topo_c, jt, f);
      }
    }
    fout[(size_t)gj * pitch + gi] = f;
    // CFL (adjust_timestep, src/timestep.h:74-87): one-sided differences
    const T du = pe - pc;
    const T dv = pn - pc;
    const auto bu = absbits_native(du), bv = absbits_native(dv);
    const auto bm = bu > bv ? bu : bv;
    mymax_n = bm > mymax_n ? bm : mymax_n;
  };
  if constexpr (sizeof(T) == 4) {
    // FP32: the Arakawa Jacobian (jacobian_lev, src/domain.h:17-27)
    // straight from the tiles, two vertically adjacent points per thread
    // sharing their 4 x 3 neighbourhoods (FP32 arithmetic is cheap; the
    // instructions that move data are not), in each 16-row band of the tile
#pragma unroll
    for (int band = 0; band < NBAND; ++band) {
    const int y0 = 16 * band + 2 * ty;
    T P[4][3], Q[4][3];
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        P[r][c] = PS(x + c - 1, y0 + r - 1);
        Q[r][c] = QS(x + c - 1, y0 + r - 1);
      }
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int y = y0 + h;
      if (EDGE && (i0 + x >= nx || j0 + y >= ny)) continue;
      const int r = h + 1;  // centre row in P, Q
      const T dxp = P[r][2] - P[r][0], dyp = P[r + 1][1] - P[r - 1][1];
      const T dxq = Q[r][2] - Q[r][0], dyq = Q[r + 1][1] - Q[r - 1][1];
      T J = dxp * dyq;
      J = fmaT(-dyp, dxq, J);
      J = fmaT(P[r][2], Q[r + 1][2] - Q[r - 1][2], J);
      J = fmaT(-P[r][0], Q[r + 1][0] - Q[r - 1][0], J);
      J = fmaT(-P[r + 1][1], Q[r + 1][2] - Q[r + 1][0], J);
      J = fmaT(P[r - 1][1], Q[r - 1][2] - Q[r - 1][0], J);
      J = fmaT(Q[r + 1][1], P[r + 1][2] - P[r + 1][0], J);
      J = fmaT(-Q[r - 1][1], P[r - 1][2] - P[r - 1][0], J);
      J = fmaT(-Q[r][2], P[r + 1][2] - P[r - 1][2], J);
      J = fmaT(Q[r][0], P[r + 1][0] - P[r - 1][0], J);
      finish(y, J, dxp, dyp, hv[2 * band + h], P[r][1], P[r][2], P[r + 1][1]);
    }
    }
  } else {
    // FP64: centred differences shared between neighbouring Jacobian
    // evaluations (fewer FP64 operations: 2 products + 8 fused terms)
    for (int w = tid; w < TY * QW; w += NT) {
      const int y = w / QW, xw = w - y * QW;
      const int xx = xw - 1;
      dyp[w] = PS(xx, y + 1) - PS(xx, y - 1);
      dyq[w] = QS(xx, y + 1) - QS(xx, y - 1);
    }
    for (int w = tid; w < QH * TX; w += NT) {
      const int y = w / TX, xw = w - y * TX;
      const int yy = y - 1;
      dxp[w] = PS(xw + 1, yy) - PS(xw - 1, yy);
      dxq[w] = QS(xw + 1, yy) - QS(xw - 1, yy);
    }
    __syncthreads();
#define DY(arr, x, y) arr[(y) * QW + (x) + 1]
#define DX(arr, x, y) arr[((y) + 1) * TX + (x)]
    for (int y = ty; y < TY; y += 8) {
      if (EDGE && (i0 + x >= nx || j0 + y >= ny)) continue;
      T J = DX(dxp, x, y) * DY(dyq, x, y);
      J = fmaT(-DY(dyp, x, y), DX(dxq, x, y), J);
      J = fmaT(PS(x + 1, y), DY(dyq, x + 1, y), J);
      J = fmaT(-PS(x - 1, y), DY(dyq, x - 1, y), J);
      J = fmaT(-PS(x, y + 1), DX(dxq, x, y + 1), J);
      J = fmaT(PS(x, y - 1), DX(dxq, x, y - 1), J);
      J = fmaT(QS(x, y + 1), DX(dxp, x, y + 1), J);
      J = fmaT(-QS(x, y - 1), DX(dxp, x, y - 1), J);
      J = fmaT(-QS(x + 1, y), DY(dyp, x + 1, y), J);
      J = fmaT(QS(x - 1, y), DY(dyp, x - 1, y), J);
      finish(y, J, DX(dxp, x, y), DY(dyp, x, y), T(0), PS(x, y), PS(x + 1, y), PS(x, y + 1));
    }
  }
#undef DY
#undef DX
#undef PS
#undef QS
  return mymax_n;
}

// End of a block's RHS work: the block's CFL maximum joins the run's
// (atomicMax on the bits), and the last of `total` blocks to finish runs
// the time-step update (adjust_timestep, src/timestep.h:74-87).
__device__ __forceinline__ void rhs_block_done(DevState* st, unsigned long long mymax, unsigned int total,
                                               double Delta, double cfl) {
  __shared__ unsigned long long wmax[NT / 32];
  __shared__ int is_last;
  const int tid = threadIdx.x + threadIdx.y * 32;
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long u = __shfl_xor_sync(0xffffffffu, mymax, o);
    mymax = u > mymax ? u : mymax;
  }
  if ((tid & 31) == 0) wmax[tid >> 5] = mymax;
  __syncthreads();
  if (tid == 0) {
    unsigned long long bm = 0ULL;
    for (int w = 0; w < NT / 32; ++w) bm = wmax[w] > bm ? wmax[w] : bm;
    atomicMax(&st->maxbits, bm);
    __threadfence();
    const unsigned int ticket = atomicAdd(&st->done_blocks, 1u);
    is_last = (ticket == total - 1);
  }
  __syncthreads();
  if (is_last && tid == 0) {
    __threadfence();
    scalar_update(st, Delta, cfl);
  }
}

// the tile at (i0, j0) plus its psi halo R touches a wall (or wraps)
__device__ __forceinline__ bool rhs_edge_tile(int i0, int j0, int R, int ty, int nx, int ny) {
  return i0 < R || j0 < R || i0 + TX + R > nx || j0 + ty + R > ny;
}

// The RHS stage of one run: tiles t = blockIdx.x, blockIdx.x + gridDim.x,
// ... over (x tile, y tile, layer).  NB >= 2 (FP32, a persistent grid): a
// ring of NB input buffers; the boxes of the tile NB - 1 iterations ahead
// are issued before the current tile is computed, so that a tile's copy has
// NB - 1 tiles' computation to arrive in.  NB == 1: one tile per block,
// loaded and then computed.
template <typename T, bool COMP, int R, int TY, int NB>
__device__ __forceinline__ void body_rhs_tiles(const StepArgs<T>& a, int ntx, int nty, unsigned char* base,
                                               const CUtensorMap* tm, unsigned long long* bar) {
  static_assert(NB >= 1 && NB <= 4, "up to four input buffers");
  DevState* st = a.state;
  if (!st->active) return;
  T* wk = rhs_work<T, R, TY>(base, NB);
  // mbarrier parities of the buffers, one bit each (a register: an array
  // indexed by the loop's buffer number would live in local memory)
  unsigned int ph = 0u;
  const int tid = threadIdx.x + threadIdx.y * 32;
  const int ntiles = ntx * nty * a.nl;
  const int si = st->step_index;
  const int step = (int)gridDim.x;
  // tile coordinates (x tile, y tile, layer) of tile t, and their advance by
  // the grid's stride without divisions (sbx < ntx and sby < nty, so one
  // carry per coordinate)
  struct TC { int bx, by, k; };
  auto tile_of = [&](int t) {
    const int r = t / ntx;
    return TC{t - r * ntx, r % nty, r / nty};
  };
  const TC sc = tile_of(step);
  auto advance = [&](TC c) {
    c.bx += sc.bx;
    const int cx = c.bx >= ntx;
    c.bx -= cx ? ntx : 0;
    c.by += sc.by + cx;
    const int cy = c.by >= nty;
    c.by -= cy ? nty : 0;
    c.k += sc.k + cy;
    return c;
  };
  // interior tiles, and closed-basin edge tiles (the box's zero fill is the
  // value outside the domain), arrive by TMA; periodic edge tiles wrap
  const bool per = a.periodic != 0;
  // the boxes of the tile at c into buffer b (thread 0)
  auto issue = [&](TC c, int b) {
    const int i1 = c.bx * TX, j1 = c.by * TY;
    if (!per || !rhs_edge_tile(i1, j1, R, TY, a.nx, a.ny))
      rhs_tile_tma<T, COMP, R, TY>(a, i1, j1, c.k, rhs_in<T, R, TY>(base, b), tm, &bar[b]);
  };
  TC cur_c = tile_of((int)blockIdx.x);
  // prologue: the block's first NB - 1 tiles into buffers 0 .. NB - 2
  if (NB >= 2 && tm && tid == 0) {
    TC c = cur_c;
    for (int p = 0; p < NB - 1; ++p, c = advance(c))
      if ((int)blockIdx.x + p * step < ntiles) issue(c, p);
  }
  // interior tiles of the compensated path's zeta mode 1 with R sweeps run
  // the compile-time form
  const bool z1 = COMP && a.zeta_mode == 1 && a.nsweep == R;
  decltype(absbits_native(T(0))) mymax = 0;
  int it = 0;
  for (int t = (int)blockIdx.x; t < ntiles; t += step, ++it, cur_c = advance(cur_c)) {
    const int cur = NB >= 2 ? it % NB : 0;
    const int i0 = cur_c.bx * TX, j0 = cur_c.by * TY, k = cur_c.k;
    const bool edge = rhs_edge_tile(i0, j0, R, TY, a.nx, a.ny);
    const RhsIn<T> in = rhs_in<T, R, TY>(base, cur);
    // the tile NB - 1 ahead into the buffer the previous tile used (every
    // thread has finished with it: the trailing __syncthreads of the
    // previous iteration)
    if (NB >= 2 && tm && tid == 0 && t + (NB - 1) * step < ntiles) {
      TC c = cur_c;
      for (int p = 0; p < NB - 1; ++p) c = advance(c);
      issue(c, (it + NB - 1) % NB);
    }
    bool ok = true;
    if (edge && (per || !tm)) {
      rhs_tile_fetch<T, COMP, R, TY, true>(a, i0, j0, k, in);
    } else if (!tm) {
      rhs_tile_fetch<T, COMP, R, TY, false>(a, i0, j0, k, in);
    } else {
      if (NB == 1 && tid == 0) rhs_tile_tma<T, COMP, R, TY>(a, i0, j0, k, in, tm, &bar[0]);
      unsigned int pb = (ph >> cur) & 1u;
      ok = rhs_tile_wait(a, &bar[cur], &pb);
      ph ^= 1u << cur;
    }
    __syncthreads();
    if (ok) {
      const auto m = edge ? rhs_tile_compute<T, COMP, R, TY, true>(a, i0, j0, k, si, in, wk)
                     : z1 ? rhs_tile_compute<T, COMP, R, TY, false, true>(a, i0, j0, k, si, in, wk)
                          : rhs_tile_compute<T, COMP, R, TY, false>(a, i0, j0, k, si, in, wk);
      mymax = m > mymax ? m : mymax;
    }
    __syncthreads();
  }
  rhs_block_done(st, widen_absbits<T>(mymax), gridDim.x, a.Delta, a.cfl);
}

// One RHS tile (bx, by, layer k) of an ensemble member, in one input
// buffer; `total` blocks share the member's CFL reduction.
template <typename T, bool COMP, int R, int TY>
__device__ __forceinline__ void body_rhs(const StepArgs<T>& a, int bx, int by, int k, unsigned int total,
                                         unsigned char* smem_raw, const CUtensorMap* tm,
                                         unsigned long long* bar, unsigned int* phase) {
  DevState* st = a.state;
  if (!st->active) return;
  const int i0 = bx * TX, j0 = by * TY;
  const bool edge = rhs_edge_tile(i0, j0, R, TY, a.nx, a.ny);
  const int si = st->step_index;
  const int tid = threadIdx.x + threadIdx.y * 32;
  const RhsIn<T> in = rhs_in<T, R, TY>(smem_raw, 0);
  T* wk = rhs_work<T, R, TY>(smem_raw, 1);
  bool ok = true;
  if (edge && (a.periodic || !tm)) {
    rhs_tile_fetch<T, COMP, R, TY, true>(a, i0, j0, k, in);
  } else if (!tm) {
    rhs_tile_fetch<T, COMP, R, TY, false>(a, i0, j0, k, in);
  } else {
    if (tid == 0) rhs_tile_tma<T, COMP, R, TY>(a, i0, j0, k, in, tm, bar);
    ok = rhs_tile_wait(a, bar, phase);
  }
  __syncthreads();
  decltype(absbits_native(T(0))) mymax = 0;
  if (ok) {
    mymax = edge ? rhs_tile_compute<T, COMP, R, TY, true>(a, i0, j0, k, si, in, wk)
                 : rhs_tile_compute<T, COMP, R, TY, false>(a, i0, j0, k, si, in, wk);
  }
  rhs_block_done(st, widen_absbits<T>(mymax), total, a.Delta, a.cfl);
}

// ------------------------------------------------------- small kernels
__device__ __forceinline__ void begin_state(DevState* st, double t_out, double tend, int max_steps) {
  st->t_out = t_out;
  st->tend = tend;
  st->first = 1;
  st->steps_taken = 0;
  st->stop_reason = 0;
  st->max_steps = max_steps;
  st->active = ((tend > 0 && !(st->t < tend)) || max_steps < 0) ? 0 : 1;
}

// work buffers of the transforms: two per row, one where the transform runs
// in place (the one-warp DST)
template <typename T>
static int dst_bufs(const StepArgs<T>& a, const DstGeom& g) {
  return (!a.periodic && !g.blue && warp_dst_len(g.H, (int)sizeof(T))) ? 1 : 2;
}
template <typename T, bool COMP>
static size_t smem_rows(const StepArgs<T>& a) {
  return cst_bytes<T>(a.nl) + (size_t)dst_bufs(a, a.gx) * a.G1 * row_len<T>(a.gx) * sizeof(T);
}
template <typename T, bool COMP>
static size_t smem_cols(const StepArgs<T>& a) {
  // periodic: two complex columns of ny values (padded rows of 2 ny reals)
  // in two or three buffers; DST: the pairs [A | C] and [B | D] of CT rows
  // ([A] and [B] without the second field)
  const bool zm = COMP && a.zeta_mode;
  const size_t rows = a.periodic ? (size_t)(zm ? 3 : 2) * 2
                                 : (size_t)(zm ? 2 : 1) * dst_bufs(a, a.gy) * col_width(a);
  return rows * row_len<T>(a.gy) * sizeof(T);
}
// column tiles of one mode: four real columns (DST) or two complex columns
// k = 0..nx/2 (periodic)
template <typename T>
static int col_tiles(const StepArgs<T>& a) {
  return a.periodic ? (a.gx.H + 2) / 2 : (a.nx + col_width(a) - 1) / col_width(a);
}
template <typename T, bool COMP>
static size_t smem_rows_inv(const StepArgs<T>& a) {
  return cst_bytes<T>(a.nl) +
         (size_t)((COMP && a.zeta_mode) ? 2 : 1) * dst_bufs(a, a.gx) * a.G3 * row_len<T>(a.gx) * sizeof(T);
}
// dynamic shared memory of the RHS kernels for halo radius r and nb input
// buffers (RhsShape)
template <typename T, int TY>
static size_t smem_rhs_rt(int r, int nb) {
  switch (r) {
    case 1: return RhsShape<T, 1, TY>::bytes(nb);
    case 2: return RhsShape<T, 2, TY>::bytes(nb);
    case 3: return RhsShape<T, 3, TY>::bytes(nb);
    default: return RhsShape<T, 4, TY>::bytes(nb);
  }
}
template <typename T>
static size_t smem_rhs_r(int r, int nb = 1, int ty = TYD) {
  return ty == 32 ? smem_rhs_rt<T, 32>(r, nb) : smem_rhs_rt<T, 16>(r, nb);
}
// halo radius of the RHS tiles: the Laplacian sweeps they run (none in zeta
// mode 2, where the whole chain is spectral), at least 1 (the Jacobian)
template <typename T>
static int rhs_halo(const StepArgs<T>& a) { return (a.nsweep > 0 && a.zeta_mode != 2) ? a.nsweep : 1; }
// the run's RHS tile height (16 or 32 rows)
template <typename T>
static int rhs_ty(const StepArgs<T>& a) { return a.rhs_ty == 32 ? 32 : 16; }
template <typename T>
static size_t smem_rhs(const StepArgs<T>& a) { return smem_rhs_r<T>(rhs_halo(a), 1, rhs_ty(a)); }
// input buffers of the single-run RHS kernel: FP32 runs its persistent
// loop on a ring of two (each tile's boxes issued one tile ahead; three,
// issued two ahead, measured the same, four cost a block per SM), FP64 one
// tile per block
template <typename T>
constexpr int rhs_nbuf() { return sizeof(T) == 4 ? 2 : 1; }
template <typename T>
static size_t smem_rhs_tiles(const StepArgs<T>& a) { return smem_rhs_r<T>(rhs_halo(a), rhs_nbuf<T>(), rhs_ty(a)); }

constexpr int RHS_RMAX = 4;  // n_hyper <= 6

}  // namespace qgw
