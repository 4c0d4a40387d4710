// GB300 (sm_103a) FDTD engine: device state, kernels and the C ABI that
// replaces the per-step operators of IrisFDTD-Academic's driver loop
// (code/driver.f90:338-451).
//
// Data layout in HBM
//   * E and H: three component arrays each, complex (double2 in FP64 mode,
//     float2 in FP32 mode), x fastest, ghost planes 0 and n+1 on every axis,
//     rows padded so that x = 1 starts on a 128-byte boundary.  The split
//     passes update them in place: the leapfrog update of a cell reads only
//     its own old value, so the reference's cur/prev pointer swap
//     (code/driver.f90:358-384) needs no second copy.  The fused pass (the
//     FP32 default) writes a second set and the two swap every step.
//   * UPML auxiliaries D and B exist for the two z slabs only, updated in
//     place (D double-buffered under the fused pass).
//   * Structure inverse permittivity over z in [hi, hf] (real when the
//     material is lossless, complex otherwise).
//   * DFT: a ring of K sample slots [K][P] gathered from the box faces after
//     each sampled step, accumulated into fdata [nof][P] (complex double)
//     one block of samples at a time.
//
// The batched form lives in iris_batch.cu, the adjoint form in
// iris_adjoint.cu; the per-cell operators they share are in iris_device.cuh,
// the fused pass's tile column in iris_fused.cuh.

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <type_traits>
#include <vector>

#include "iris_engine.h"
#include "iris_fused.cuh"

namespace iris {
namespace {

template <typename T, bool CEPS>
__global__ void __launch_bounds__(256) k_update_e(FieldArgs<T> a) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int y = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int z = blockIdx.z * blockDim.z + threadIdx.z + 1;
  if (x > a.g.nx || y > a.g.ny || z > a.g.nz) return;
  e_split_cell<T, CEPS>(a, x, y, z);
}

template <typename T>
__global__ void __launch_bounds__(256) k_update_h(FieldArgs<T> a) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int y = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int z = blockIdx.z * blockDim.z + threadIdx.z + 1;
  if (x > a.g.nx || y > a.g.ny || z > a.g.nz) return;
  h_split_cell<T>(a, x, y, z);
}

// The device-resident step base of captured graphs.
__global__ void k_set_int(int* p, int v) { *p = v; }
__global__ void k_add_int(int* p, int v) { *p += v; }

// ---------------------------------------------------------------------------
// Streamed split passes (FP32, real material).
//
// A CTA owns an SX x SY column tile of one cell and marches z over a chunk of
// up to SZC planes.  Each plane a pass reads is staged in shared memory by
// 1-D bulk copies (cp.async.bulk: the TMA engine, issued by one warp, one
// copy per row and component) into a ring of SNST stage buffers, each with an
// mbarrier that completes when its bytes have landed; the next two planes
// are in flight while one is computed.  Rows are copied from 16-byte aligned
// starts (x = 1 sits on a 128-byte boundary, SX is a multiple of 4) and
// trimmed to the cells the tile needs, so DRAM traffic stays at the
// algorithmic bytes.  The arithmetic is that of the split passes.

constexpr int SX = 32, SY = 8, SNST = 4, SZC = 32;

struct StageE {                 // E pass, plane z
  float2 h[3][SY + 1][SX + 2];  // H rows y0-1 .. y0+SY-1, cells x0-2 .. x0+SX-1
  float2 e[3][SY][SX];          // E rows y0 .. y0+SY-1, cells x0 .. x0+SX-1
  float eps[SY][SX];            // structure eps_inv (planes hi..hf)
};
struct StageH {                 // H pass, plane z
  float2 e[3][SY + 1][SX + 2];  // E rows y0 .. y0+SY, cells x0 .. x0+SX+1
  float2 h[3][SY][SX];          // H rows y0 .. y0+SY-1, cells x0 .. x0+SX-1
};
static_assert(sizeof(StageE) % 16 == 0 && sizeof(StageH) % 16 == 0, "stage buffers keep 16-byte alignment");
constexpr size_t STREAM_SMEM_E = SNST * sizeof(StageE);
constexpr size_t STREAM_SMEM_H = SNST * sizeof(StageH);


__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Waits for phase parity of bar for at most about limit clock cycles;
// false when it gave up.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity, long long limit) {
  if (mbar_try_wait(bar, parity)) return true;
  const long long t0 = clock64();
  while (!mbar_try_wait(bar, parity))
    if (clock64() - t0 > limit) return false;
  return true;
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

constexpr long long STREAM_WAIT_CYCLES = 1LL << 31;  // about a second

// IRIS_OP_WAIT_CHECK: an mbarrier armed for 16 bytes that no copy delivers,
// waited on with the streamed passes' limit divided by 2^shift; the give-up
// is recorded (code 4) as the passes record theirs.
__global__ void k_wait_check(int* err, int shift) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x != 0) return;
  mbar_init(&bar, 1);
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  mbar_expect_tx(&bar, 16);
  if (!mbar_wait(&bar, 0, STREAM_WAIT_CYCLES >> shift)) atomicExch(err, 4);
}

// Issue (warp 0) the bulk copies of plane z into stage S of the E pass:
// full: H (3 components, rows y0-1 .. y0+nye-1), E (3 components, own rows)
// and, on structure planes, eps_inv; otherwise H components 1, 2 of the own
// rows (the plane below the chunk).
__device__ __forceinline__ void stream_issue_e(const FieldArgs<float>& a, StageE* S, uint64_t* bar, int x0, int y0,
                                               int z, bool full) {
  const Geo& g = a.g;
  const int lane = threadIdx.x;
  const int nxe = min(SX, g.nx - x0 + 1), nye = min(SY, g.ny - y0 + 1);
  const unsigned bh = (unsigned)((nxe + 3) & ~1) * 8u;  // cells x0-2 .. x0+nxe-1
  const unsigned be = (unsigned)((nxe + 1) & ~1) * 8u;  // cells x0 .. x0+nxe-1
  const unsigned bp = (unsigned)((nxe + 3) & ~3) * 4u;
  const bool ep = full && z >= a.hi && z <= a.hf;
  const int nh = full ? 3 * (nye + 1) : 2 * nye, ne = full ? 3 * nye : 0, np = ep ? nye : 0;
  if (lane == 0) mbar_expect_tx(bar, nh * bh + ne * be + np * bp);
  __syncwarp();
  fence_proxy_async();
  for (int q = lane; q < nh + ne + np; q += 32) {
    if (q < nh) {
      const int k = full ? q / (nye + 1) : q / nye;
      const int r = full ? q % (nye + 1) : 1 + q % nye;
      bulk_g2s(&S->h[k][r][0], a.h + k * g.comp + g.at(x0 - 2, y0 - 1 + r, z), bh, bar);
    } else if (q < nh + ne) {
      const int k = (q - nh) / nye, r = (q - nh) % nye;
      bulk_g2s(&S->e[k][r][0], a.e + k * g.comp + g.at(x0, y0 + r, z), be, bar);
    } else {
      const int r = q - nh - ne;
      bulk_g2s(&S->eps[r][0], a.eps_r + (long)(z - a.hi) * g.plane + g.at(x0, y0 + r, 0), bp, bar);
    }
  }
}

// Issue (warp 0) the bulk copies of plane z into stage S of the H pass:
// full: E (3 components, rows y0 .. y0+nye, cells x0 .. x0+nxe) and H (own
// rows and cells); otherwise E components 1, 2 of the own rows and cells
// (the plane above the chunk).
__device__ __forceinline__ void stream_issue_h(const FieldArgs<float>& a, StageH* S, uint64_t* bar, int x0, int y0,
                                               int z, bool full) {
  const Geo& g = a.g;
  const int lane = threadIdx.x;
  const int nxe = min(SX, g.nx - x0 + 1), nye = min(SY, g.ny - y0 + 1);
  const unsigned bx = (unsigned)((nxe + 2) & ~1) * 8u;  // cells x0 .. x0+nxe
  const unsigned bo = (unsigned)((nxe + 1) & ~1) * 8u;  // cells x0 .. x0+nxe-1
  const int ne = full ? 3 * (nye + 1) : 2 * nye, nh = full ? 3 * nye : 0;
  if (lane == 0) mbar_expect_tx(bar, full ? ne * bx + nh * bo : ne * bo);
  __syncwarp();
  fence_proxy_async();
  for (int q = lane; q < ne + nh; q += 32) {
    if (q < ne) {
      const int k = full ? q / (nye + 1) : q / nye;
      const int r = full ? q % (nye + 1) : q % nye;
      bulk_g2s(&S->e[k][r][0], a.e + k * g.comp + g.at(x0, y0 + r, z), full ? bx : bo, bar);
    } else {
      const int k = (q - ne) / nye, r = (q - ne) % nye;
      bulk_g2s(&S->h[k][r][0], a.h + k * g.comp + g.at(x0, y0 + r, z), bo, bar);
    }
  }
}

// Bounded wait for every stage still being filled (after a failed wait).
__device__ __forceinline__ void stream_drain(uint64_t* bar, unsigned par, unsigned pend) {
  for (int s = 0; s < SNST; ++s)
    if (pend & (1u << s)) mbar_wait(bar + s, (par >> s) & 1u, STREAM_WAIT_CYCLES >> 4);
}

// The E pass over planes zs .. min(zs+SZC-1, nz) of the tile at (x0, y0).
// par: expected phase parity per stage, block-uniform, carried across tiles.
// Returns false when a stage never completed (*err is then set).
__device__ bool stream_tile_e(const FieldArgs<float>& a, int x0, int y0, int zs, StageE* S, uint64_t* bar,
                              unsigned& par, int* err) {
  const Geo& g = a.g;
  const int ze = min(zs + SZC - 1, g.nz);
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int x = x0 + tx, y = y0 + ty;
  const bool own = x <= g.nx && y <= g.ny;
  const bool w0 = ty == 0;
  unsigned pend = 0;
  // ring slot of plane p: (p - zs + 1) % SNST
  if (w0) {
    stream_issue_e(a, S + 0, bar + 0, x0, y0, zs - 1, false);
    stream_issue_e(a, S + 1, bar + 1, x0, y0, zs, true);
    if (zs + 1 <= ze) stream_issue_e(a, S + 2, bar + 2, x0, y0, zs + 1, true);
  }
  pend = zs + 1 <= ze ? 7u : 3u;
  bool bad = false;
  for (int z = zs; z <= ze; ++z) {
    const int j = z - zs;
    if (z + 2 <= ze) {
      if (w0) stream_issue_e(a, S + (j + 3) % SNST, bar + (j + 3) % SNST, x0, y0, z + 2, true);
      pend |= 1u << ((j + 3) % SNST);
    }
    if (j == 0) {
      bad |= !mbar_wait(bar, par & 1u, STREAM_WAIT_CYCLES);
      par ^= 1u;
      pend &= ~1u;
    }
    const int c = (j + 1) % SNST, pv = j % SNST;
    bad |= !mbar_wait(bar + c, (par >> c) & 1u, STREAM_WAIT_CYCLES);
    par ^= 1u << c;
    pend &= ~(1u << c);
    if (own) {
      const StageE& C = S[c];
      const StageE& P = S[pv];
      const float2 a0 = C.h[0][ty + 1][tx + 2], a1 = C.h[1][ty + 1][tx + 2], a2 = C.h[2][ty + 1][tx + 2];
      const cx<float> h0{a0.x, a0.y}, h1{a1.x, a1.y}, h2{a2.x, a2.y};
      auto f = [](float2 v) { return cx<float>{v.x, v.y}; };
      cx<float> cu[3], e[3];
      cu[0] = cadd(csub(csub(h2, f(C.h[2][ty][tx + 2])), h1), f(P.h[1][ty + 1][tx + 2]));
      cu[1] = cadd(csub(csub(h0, f(P.h[0][ty + 1][tx + 2])), h2), f(C.h[2][ty + 1][tx + 1]));
      cu[2] = cadd(csub(csub(h1, f(C.h[1][ty + 1][tx + 1])), h0), f(C.h[0][ty][tx + 2]));
#pragma unroll
      for (int k = 0; k < 3; ++k) e[k] = f(C.e[k][ty][tx]);
      e_apply<float, false, 7, true>(a, a.pml_d, x, y, z, cu, e, C.eps[ty][tx]);
      const long i = g.at(x, y, z);
#pragma unroll
      for (int k = 0; k < 3; ++k) st<float>(a.e + k * g.comp + i, e[k]);
      if (x == 1) {
        const long q = g.at(g.nx + 1, y, z);
#pragma unroll
        for (int k = 0; k < 3; ++k) st<float>(a.e + k * g.comp + q, cmul(a.pxp, e[k]));
      }
      if (y == 1) {
        const long q = g.at(x, g.ny + 1, z);
#pragma unroll
        for (int k = 0; k < 3; ++k) st<float>(a.e + k * g.comp + q, cmul(a.pyp, e[k]));
      }
      if (z == 1) {
        const long q = g.at(x, y, g.nz + 1);
#pragma unroll
        for (int k = 0; k < 3; ++k) st<float>(a.e + k * g.comp + q, cmul(a.pzp, e[k]));
      }
    }
    if (__syncthreads_or(bad)) {
      if (threadIdx.x == 0 && threadIdx.y == 0) atomicExch(err, 1);
      stream_drain(bar, par, pend);
      return false;
    }
  }
  return true;
}

// The H pass over planes zs .. min(zs+SZC-1, nz) of the tile at (x0, y0).
__device__ bool stream_tile_h(const FieldArgs<float>& a, int x0, int y0, int zs, StageH* S, uint64_t* bar,
                              unsigned& par, int* err) {
  const Geo& g = a.g;
  const int ze = min(zs + SZC - 1, g.nz);
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int x = x0 + tx, y = y0 + ty;
  const bool own = x <= g.nx && y <= g.ny;
  const bool w0 = ty == 0;
  // ring slot of plane p: (p - zs) % SNST; plane ze+1 is partial
  unsigned pend = 0;
  for (int p = zs; p <= min(zs + 2, ze + 1); ++p) {
    if (w0) stream_issue_h(a, S + (p - zs), bar + (p - zs), x0, y0, p, p <= ze);
    pend |= 1u << (p - zs);
  }
  bool bad = false;
  for (int z = zs; z <= ze; ++z) {
    const int j = z - zs;
    if (z + 3 <= ze + 1) {
      if (w0) stream_issue_h(a, S + (j + 3) % SNST, bar + (j + 3) % SNST, x0, y0, z + 3, z + 3 <= ze);
      pend |= 1u << ((j + 3) % SNST);
    }
    if (j == 0) {
      bad |= !mbar_wait(bar, par & 1u, STREAM_WAIT_CYCLES);
      par ^= 1u;
      pend &= ~1u;
    }
    const int c = j % SNST, n = (j + 1) % SNST;
    bad |= !mbar_wait(bar + n, (par >> n) & 1u, STREAM_WAIT_CYCLES);
    par ^= 1u << n;
    pend &= ~(1u << n);
    if (own) {
      const StageH& C = S[c];
      const StageH& N = S[n];
      auto f = [](float2 v) { return cx<float>{v.x, v.y}; };
      cx<float> ev[3], xp[3], yp[3], zp[3], h[3];
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        ev[k] = f(C.e[k][ty][tx]);
        h[k] = f(C.h[k][ty][tx]);
      }
      xp[1] = f(C.e[1][ty][tx + 1]);
      xp[2] = f(C.e[2][ty][tx + 1]);
      yp[0] = f(C.e[0][ty + 1][tx]);
      yp[2] = f(C.e[2][ty + 1][tx]);
      zp[0] = f(N.e[0][ty][tx]);
      zp[1] = f(N.e[1][ty][tx]);
      h_update<float>(a, x, y, z, ev, xp, yp, zp, h);
      const long i = g.at(x, y, z);
#pragma unroll
      for (int k = 0; k < 3; ++k) st<float>(a.h + k * g.comp + i, h[k]);
      if (x == g.nx) {
        const long q = g.at(0, y, z);
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          st<float>(a.e + k * g.comp + q, cmul(a.pxm, ev[k]));
          st<float>(a.h + k * g.comp + q, cmul(a.pxm, h[k]));
        }
      }
      if (y == g.ny) {
        const long q = g.at(x, 0, z);
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          st<float>(a.e + k * g.comp + q, cmul(a.pym, ev[k]));
          st<float>(a.h + k * g.comp + q, cmul(a.pym, h[k]));
        }
      }
      if (z == g.nz) {
        const long q = g.at(x, y, 0);
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          st<float>(a.e + k * g.comp + q, cmul(a.pzm, ev[k]));
          st<float>(a.h + k * g.comp + q, cmul(a.pzm, h[k]));
        }
      }
    }
    if (__syncthreads_or(bad)) {
      if (threadIdx.x == 0 && threadIdx.y == 0) atomicExch(err, 2);
      stream_drain(bar, par, pend);
      return false;
    }
  }
  return true;
}

__device__ __forceinline__ void stream_init(uint64_t* bar) {
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    for (int s = 0; s < SNST; ++s) mbar_init(bar + s, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
}

// One engine: grid (ceil(nx/SX), ceil(ny/SY), ceil(nz/SZC)), block (SX, SY).
__global__ void __launch_bounds__(SX* SY) k_stream_e(FieldArgs<float> a, int* err) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ uint64_t bar[SNST];
  stream_init(bar);
  unsigned par = 0;
  stream_tile_e(a, 1 + blockIdx.x * SX, 1 + blockIdx.y * SY, 1 + blockIdx.z * SZC, (StageE*)smem, bar, par, err);
}

__global__ void __launch_bounds__(SX* SY) k_stream_h(FieldArgs<float> a, int* err) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ uint64_t bar[SNST];
  stream_init(bar);
  unsigned par = 0;
  stream_tile_h(a, 1 + blockIdx.x * SX, 1 + blockIdx.y * SY, 1 + blockIdx.z * SZC, (StageH*)smem, bar, par, err);
}

template <typename T>
// The step is it, or *itp + it when itp is given (a device-resident step
// base, which lets a captured graph of steps be replayed at any step).
__global__ void __launch_bounds__(64) k_tfsf(typename V2<T>::t* e, typename V2<T>::t* h, Geo g, SrcArgs s, int it,
                                             const int* itp) {
  const int ix = blockIdx.x * blockDim.x + threadIdx.x;
  if (ix > s.nx + 1) return;
  if (itp) it += *itp;
  const int y0 = blockIdx.y * TFSF_YCH;
  tfsf_column<T>(e, h, g, s, it, ix, y0, min(y0 + TFSF_YCH - 1, s.ny + 1));
}


template <typename T>
__global__ void __launch_bounds__(256) k_dft_gather(const typename V2<T>::t* __restrict__ e,
                                                    const typename V2<T>::t* __restrict__ h, long comp,
                                                    const Seg* __restrict__ segs, typename V2<T>::t* __restrict__ slot,
                                                    int* tk, int islot, int t, const int* tp, long np) {
  if (blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0) tk[islot] = tp ? *tp + t : t;
  const Seg sg = segs[blockIdx.y];
  const typename V2<T>::t* src = sg.field < 3 ? e + sg.field * comp : h + (sg.field - 3) * comp;
  gather_run<T>(sg, src, slot, comp, np);
}

// FP64 mode: fdata(p, iw) += (dt*F_k(p))*exp(i*fw(iw)*t_k), k in the
// reference's order (code/dataprocess.f90:143-147), each complex
// multiply-add as four FP64 FMAs (GB300's FP64 rate makes the unfused eight
// operations the cost of the FP64 mode; the difference is one rounding per
// term).  The twiddles exp(i*fw*t_k) come from one table per block.
constexpr int DFT64_WC = 8;
__global__ void k_twiddle64(const int* __restrict__ tk, int nk, const double* __restrict__ fw, int nof,
                            double2* __restrict__ W) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nk * nof) return;
  const int k = t / nof, j = t % nof;
  double sn, cs;
  sincos(dm(fw[j], (double)tk[k]), &sn, &cs);
  W[t] = make_double2(cs, sn);
}

__global__ void __launch_bounds__(128) k_dft_fp64(const double2* __restrict__ S, long P, int nk,
                                                  const double2* __restrict__ W, int nof, int nwc, double dt,
                                                  double2* __restrict__ fd) {
  extern __shared__ double2 W64[];  // [nk][WC]
  // 1-D grid, frequency chunks fastest: the chunks of one point block share its samples in L2
  const int w0 = (blockIdx.x % nwc) * DFT64_WC;
  const long pblk = blockIdx.x / nwc;
  for (int t = threadIdx.x; t < nk * DFT64_WC; t += blockDim.x) {
    const int k = t / DFT64_WC, j = t % DFT64_WC;
    W64[t] = w0 + j < nof ? W[(long)k * nof + w0 + j] : make_double2(0.0, 0.0);
  }
  __syncthreads();
  const long p = pblk * blockDim.x + threadIdx.x;
  if (p >= P) return;
  const int nw = min(DFT64_WC, nof - w0);
  double2 acc[DFT64_WC];
#pragma unroll
  for (int j = 0; j < DFT64_WC; ++j)
    if (j < nw) acc[j] = fd[(long)(w0 + j) * P + p];
  for (int k = 0; k < nk; ++k) {
    const double2 f = S[(long)k * P + p];
    const double ar = dm(dt, f.x), ai = dm(dt, f.y);
#pragma unroll
    for (int j = 0; j < DFT64_WC; ++j) {
      const double2 w = W64[k * DFT64_WC + j];
      acc[j].x = fma(ar, w.x, fma(-ai, w.y, acc[j].x));
      acc[j].y = fma(ar, w.y, fma(ai, w.x, acc[j].y));
    }
  }
#pragma unroll
  for (int j = 0; j < DFT64_WC; ++j)
    if (j < nw) fd[(long)(w0 + j) * P + p] = acc[j];
}

// FP32 mode accumulators: each complex value of fdata is a compensated
// (double-float) pair per part, float4 (re_hi, im_hi, re_lo, im_lo), 16 bytes
// like a double2.  GB300 runs FP64 arithmetic at a small fraction of its FP32
// rate, and the block accumulation and the flux read add to every stored
// value: in FP64 those adds and the float-to-double conversions bound both
// kernels, in FP32 they cost nothing next to the memory traffic.  A partial
// sum p is added by TwoSum (hi + p exactly as s + e), the error term joins
// lo, and the pair is renormalised (Fast2Sum): hi + lo carries about 48
// bits.
__device__ __forceinline__ void df_add(float& hi, float& lo, float p) {
  const float s = __fadd_rn(hi, p);
  const float bp = __fsub_rn(s, hi);
  const float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bp)), __fsub_rn(p, bp));
  const float t = __fadd_rn(lo, e);
  const float h = __fadd_rn(s, t);
  lo = __fsub_rn(t, __fsub_rn(h, s));
  hi = h;
}
// The accumulator types: double2 (FP64 accumulation) and float4 (double-float).
__device__ __forceinline__ void acc_add(double2& a, float re, float im) {
  a.x += (double)re;
  a.y += (double)im;
}
__device__ __forceinline__ void acc_add(float4& a, float re, float im) {
  df_add(a.x, a.z, re);
  df_add(a.y, a.w, im);
}
// The leading part df_add leaves in hi, without the new lo (a flux read uses
// the leading parts only and stores nothing): the same operations up to hi.
__device__ __forceinline__ float df_add_hi(float hi, float lo, float p) {
  const float s = __fadd_rn(hi, p);
  const float bp = __fsub_rn(s, hi);
  const float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bp)), __fsub_rn(p, bp));
  return __fadd_rn(s, __fadd_rn(lo, e));
}
// v * 2^e2 as a double, formed from the float's bits with integer operations
// only (exact for |e2| well inside the double range; GB300's FP64 pipe is
// kept out of the flux epilogue).  A zero stays a signed zero, Inf and NaN
// stay Inf and NaN, a subnormal v is normalised by its leading bit.
__device__ __forceinline__ double scaled_double(float v, int e2) {
  const unsigned u = __float_as_uint(v);
  const unsigned long long sign = (unsigned long long)(u >> 31) << 63;
  const unsigned ef = (u >> 23) & 0xffu;
  unsigned long long m = u & 0x7fffffu;
  if (ef == 0xffu) return __longlong_as_double((long long)(sign | (0x7ffull << 52) | (m << 29)));
  int e = (int)ef - 127;
  if (ef == 0u) {
    if (m == 0u) return __longlong_as_double((long long)sign);
    // subnormal: m * 2^-149, normalised by its leading bit
    const int top = 31 - __clz((int)m);  // 0 .. 22
    e = top - 149;
    m = (m << (23 - top)) & 0x7fffffull;
  }
  return __longlong_as_double((long long)(sign | ((unsigned long long)(e + 1023 + e2) << 52) | (m << 29)));
}

// Value of an accumulator in FP64.
__device__ __forceinline__ double2 acc_value(const double2& a) { return a; }
__device__ __forceinline__ double2 acc_value(const float4& a) {
  return make_double2((double)a.x + (double)a.z, (double)a.y + (double)a.w);
}

// FP32 mode twiddles: Wt[k][iw] = dt*exp(i*fw(iw)*t_k), phase formed in FP64
// (it reaches ~1e4 rad), rounded to FP32 once.
// Time index of sample k: tk[k], or t0 + k*tstep when tk is null.
__global__ void k_twiddle(const int* __restrict__ tk, int t0, int tstep, int nk, const double* __restrict__ fw,
                          int nof, double dt, float2* __restrict__ Wt) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nk * nof) return;
  const int k = t / nof, j = t % nof;
  const int tt = tk ? tk[k] : t0 + k * tstep;
  double sn, cs;
  sincos(fw[j] * (double)tt, &sn, &cs);
  Wt[t] = make_float2((float)(dt * cs), (float)(dt * sn));
}

// FP32 mode: partial[p][iw] = sum_k F_k(p)*Wt[k][iw] in FP32 registers over
// the block of nk samples, then one add per (p, iw) into fdata (double-float
// in the engine, FP64 accumulators for iris_dft_block_noalloc's callers).
// CTA tile: 128 points x 32 frequencies, 128 threads (three CTAs per SM, so one
// CTA's staging overlaps the others' FMAs).  Lane l owns points l + 32 i
// (i < 4), warp w owns frequencies 8 w + j (j < 8), so each thread keeps a
// 4 x 8 complex register tile and every k costs 8 shared loads for 128 FMAs.
// Samples and twiddles are staged through shared memory 32 k at a time.  The
// 1-D grid runs the frequency chunks of one point tile back to back so the
// tile's samples are read from HBM once and from L2 after that.
constexpr int DFT_TP = 128, DFT_TW = 32, DFT_KC = 32, DFT_THREADS = 128;
template <typename ACC>
__global__ void __launch_bounds__(DFT_THREADS) k_dft_fp32(const float2* __restrict__ S, long P, int nk,
                                                  const float2* __restrict__ Wt, int nof, int nwc,
                                                  ACC* __restrict__ fd) {
  __shared__ float2 Ss[DFT_KC][DFT_TP];
  __shared__ float4 Ws[DFT_KC][DFT_TW / 2];
  const int wc = blockIdx.x % nwc;
  const long p0 = (long)(blockIdx.x / nwc) * DFT_TP;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  float ar[4][8], ai[4][8];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 8; ++j) ar[i][j] = ai[i][j] = 0.f;
  for (int kc = 0; kc < nk; kc += DFT_KC) {
    const int kn = min(DFT_KC, nk - kc);
    for (int t = threadIdx.x; t < kn * DFT_TP; t += blockDim.x) {
      const int k = t / DFT_TP, q = t % DFT_TP;
      const long p = p0 + q;
      Ss[k][q] = p < P ? S[(long)(kc + k) * P + p] : make_float2(0.f, 0.f);
    }
    for (int t = threadIdx.x; t < kn * (DFT_TW / 2); t += blockDim.x) {
      const int k = t / (DFT_TW / 2), j2 = t % (DFT_TW / 2);
      const int w = wc * DFT_TW + 2 * j2;
      const float2 a = w < nof ? Wt[(long)(kc + k) * nof + w] : make_float2(0.f, 0.f);
      const float2 b = w + 1 < nof ? Wt[(long)(kc + k) * nof + w + 1] : make_float2(0.f, 0.f);
      Ws[k][j2] = make_float4(a.x, a.y, b.x, b.y);
    }
    __syncthreads();
    for (int k = 0; k < kn; ++k) {
      float2 sv[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) sv[i] = Ss[k][lane + 32 * i];
      float wr[8], wi[8];
#pragma unroll
      for (int j2 = 0; j2 < 4; ++j2) {
        const float4 w = Ws[k][warp * 4 + j2];
        wr[2 * j2] = w.x;
        wi[2 * j2] = w.y;
        wr[2 * j2 + 1] = w.z;
        wi[2 * j2 + 1] = w.w;
      }
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          ar[i][j] = fmaf(sv[i].x, wr[j], fmaf(-sv[i].y, wi[j], ar[i][j]));
          ai[i][j] = fmaf(sv[i].x, wi[j], fmaf(sv[i].y, wr[j], ai[i][j]));
        }
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const long p = p0 + lane + 32 * i;
    if (p >= P) continue;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int w = wc * DFT_TW + warp * 8 + j;
      if (w >= nof) continue;
      ACC* q = fd + (long)w * P + p;
      ACC f = *q;
      acc_add(f, ar[i][j], ai[i][j]);
      *q = f;
    }
  }
}

// ---------------------------------------------------------------------------
// FP32 DFT block on the tensor cores (tcgen05.mma kind::tf32).
//
// fdata[iw][p] += sum_k F_k(p) W_k(iw), W_k(iw) = dt exp(i fw(iw) t_k), for a
// block of nk samples is the real GEMM C = A B with
//   A[p][2k+c]      = Re (c = 0) / Im (c = 1) of F_k(p)       M = points
//   B[2k+c][2j+d]   = the real 2x2 form of W_k(iw0 + j)       N = 2 x frequencies
// so that C[p][2j] and C[p][2j+1] are Re and Im of the (p, iw0+j) partial sum.
// FP32 accuracy from TF32 operands: with X = Xh + Xl, Xh = X rounded to TF32,
// A B ~ Ah Bh + Ah Bl + Al Bh (the Al Bl term is below FP32 rounding).
//
// A work item is a row tile of TC_M = 128 sample points (the 128 TMEM lanes)
// and a group of up to TC_NW = 128 frequencies (256 FP32 TMEM columns).  K
// is walked in chunks of TC_KC = 16 (8 samples): the A operands split into
// hi/lo (K-major core matrices, no swizzle) in shared memory, the B
// operands, identical for every item of a group, prepared once per block in
// global memory in the same layout by k_twiddle_tc and bulk-copied (TMA) per
// chunk.  The kernels are k_dft_ws_commit and k_dft_ws_flux below.

constexpr int TC_M = 128, TC_NW = 128, TC_KC = 16;
constexpr int TC_NMAX = 2 * TC_NW;                       // TMEM columns per CTA
constexpr int TC_BROWS = TC_NMAX;                        // B rows per chunk buffer
constexpr size_t TC_A_BYTES = (size_t)TC_M * TC_KC * 4;  // one of A hi / A lo
constexpr size_t TC_B_BYTES = (size_t)TC_BROWS * TC_KC * 4;
constexpr size_t TC_STAGE = 2 * TC_A_BYTES + 2 * TC_B_BYTES;

// Offset (in floats) of element (row r, k) of a K-major, unswizzled operand
// of TC_KC columns: 8-row x 16-byte core matrices, the K-neighbour core
// matrix 128 bytes on, the next 8-row group TC_KC/4 core matrices on.
__host__ __device__ __forceinline__ int tc_off(int r, int k) {
  return ((r >> 3) * (TC_KC / 4) + (k >> 2)) * 32 + (r & 7) * 4 + (k & 3);
}

__device__ __forceinline__ float tf32_hi(float x) {
  unsigned u;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(u) : "f"(x));
  return __uint_as_float(u);
}

// B operands of every frequency group and chunk of one block, hi then lo:
// Bt[((g * nch + c) * 2 + h) * TC_BROWS * TC_KC + tc_off(n, kk)].
__global__ void k_twiddle_tc(const int* __restrict__ tk, int t0, int tstep, int nk, const double* __restrict__ fw,
                             int nof, double dt, int ngroups, int nch, float* __restrict__ Bt) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const long per = (long)TC_BROWS * TC_KC;
  if (t >= (long)ngroups * nch * per) return;
  const int g = (int)(t / (nch * per)), c = (int)((t / per) % nch);
  const int n = (int)((t % per) / TC_KC), kk = (int)(t % TC_KC);
  const int j = n >> 1, d = n & 1, iw = g * TC_NW + j;
  const int k2 = c * TC_KC + kk, k = k2 >> 1, cc = k2 & 1;
  float v = 0.f;
  if (iw < nof && k < nk) {
    const int tt = tk ? tk[k] : t0 + k * tstep;
    double sn, cs;
    sincos(fw[iw] * (double)tt, &sn, &cs);
    const float wr = (float)(dt * cs), wi = (float)(dt * sn);
    v = d == 0 ? (cc == 0 ? wr : -wi) : (cc == 0 ? wi : wr);
  }
  const float hi = tf32_hi(v);
  float* base = Bt + ((long)(g * nch + c) * 2) * per;
  base[tc_off(n, kk)] = hi;
  base[per + tc_off(n, kk)] = v - hi;
}

__device__ __forceinline__ uint64_t tc_desc(const void* smem) {
  // start address, leading (K) byte offset 128, stride (8-row) byte offset
  // TC_KC/4 * 128, descriptor version 1, no swizzle
  const uint64_t a = (smem_u32(smem) & 0x3FFFFu) >> 4;
  const uint64_t lbo = 128u >> 4, sbo = (uint64_t)(TC_KC / 4 * 128) >> 4;
  return a | (lbo << 16) | (sbo << 32) | (1ull << 46);
}

// kind::tf32, D = F32, A = B = TF32, both K-major, M = 128, N = n.
__host__ __device__ constexpr uint32_t tc_idesc(int n) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(TC_M >> 4) << 24);
}

__device__ __forceinline__ void tc_mma(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, int acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(acc)
      : "memory");
}
__device__ __forceinline__ void tc_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

// ---------------------------------------------------------------------------
// Flux read without committing the sample ring (FP32 mode, tensor cores).
//
// For face f and frequency iw, the Jabs of scattering_fourier_out
// (code/dataprocess.f90:246-277) over the accumulators as they would stand
// after a commit of the nk samples still in the ring:
//   J = sign * scale * sum_L Re(A_a conj A_b) - Re(A_c conj A_d),
//   A_x(L, iw) = fdata[iw][p_x + L] + sum_k F_k(p_x + L) Wt_k(iw).
// The pending sum is the commit's block GEMM (the same MMAs on the same
// operands, so each A_x is the value a commit would store), but nothing is
// written back: a flux read costs one read of the four flux components'
// accumulators, and the ring is committed when it is full, as before.  Its
// work items are tiles of FL_LOC = 32 locations of one face (k_dft_ws_flux,
// flux mode); k_flux_sum adds the partials of a face in a fixed order, so
// the result does not depend on scheduling.
constexpr int FL_LOC = 32;

struct FluxTiles {
  int start[7];  // first tile of face f; start[6]: tiles of the set
};

__device__ __forceinline__ long face_comp(const FluxFace& F, int c) {
  return c == 0 ? F.pa : c == 1 ? F.pb : c == 2 ? F.pc : F.pd;
}

// ---------------------------------------------------------------------------
// Warp-specialised persistent DFT block kernel (FP32 mode, tensor cores).
//
// One CTA per SM walks work items (a row tile and a frequency group) with
// three roles that overlap each other through mbarriers (the per-mode warp
// counts and prefetch depths are WsCfg's, below):
//   * producer warps: the samples of a chunk of 8 samples into the TF32
//     hi/lo A operands of a stage (plain loads, held some chunks ahead in
//     registers), and one thread bulk-copies the chunk's B operands into the
//     same stage; WS_STAGES stages in a ring.  Shared memory stays at the
//     three stages: what more it takes comes out of the L1, which holds the
//     loads in flight (a raw sample ring in shared memory fed by
//     asynchronous copies left 20 KB of L1 and made both modes 1.3 to 1.8
//     times slower);
//   * the MMA thread (the last warp): three tcgen05.mma kind::tf32 per 8 K
//     columns into one of two TMEM accumulators (256 columns each), each
//     stage freed by a commit when its MMAs are done, each finished item
//     signalled by a commit on that accumulator;
//   * epilogue warps (warp w reads TMEM lanes 32 (w % 4), the four warps of a
//     group cover the four lane quarters, group k of NG takes the 4-frequency
//     chunks k, k + NG, ...): drain an accumulator while the MMAs of the next
//     item fill the other, streaming the accumulators ahead in registers.
//     Many warps, because the epilogue's work per value (the double-float
//     update, the products and their shuffles) needs more warps in flight
//     than its memory stream alone would.
// Commit mode: rows are 128 consecutive sample points; the epilogue adds the
// partial sums into fdata (read once, written once).
// Flux mode: rows are the four flux components of 32 locations of one face,
// row 32 q + 4 l + c = component c of location 8 q + l, so that the warp
// reading TMEM lane quarter q holds all four components of its 8 locations;
// the epilogue adds the partial sums to the accumulators it reads, forms the
// face's products with shuffles inside the warp and writes one partial per
// (frequency, tile, quarter); fdata is not written.  No barrier spans
// warps, so a warp that gives up leaves no other waiting for it.
// Every wait is bounded: a role that gives up records it (code 3 in commit
// mode, 5 in flux mode) and stops; the others stop at their next wait; the
// CTA waits (bounded) for its copies and MMAs before it frees its TMEM.

constexpr int WS_STAGES = 3, WS_FCH = 4;
constexpr size_t WS_SMEM = WS_STAGES * TC_STAGE;
// Per-mode layout.  A sub-partition holds a quarter of the register file, and
// the warps of a CTA are dealt to the four in turn, so W warps of R registers
// fit when ceil(W / 4) x 32 x R <= 16384.  Commit mode (the A stream is the
// whole sample ring): eight producer warps, each thread half a row (4 of a
// chunk's 8 samples), three chunks ahead in registers (one chunk ahead on two
// warps left 8 KB of sample loads in flight per SM and the producers
// latency-bound; two ahead on four warps measured 9 % slower than this, four
// ahead 3-7 % slower), and twelve epilogue warps streaming the accumulators
// two chunks ahead (4 % faster than sixteen one chunk ahead); 21 warps, 80
// registers.  Flux mode
// (a few buffered samples, the accumulators dominate): two producer warps,
// two rows a thread, one chunk ahead; 19 warps, 96 registers for the
// epilogue's products (twelve epilogue warps streaming two chunks ahead, 15
// warps at 128 registers, measured 1.13-1.17 times slower: the flux epilogue
// is bound by instruction issue more than by loads in flight).
template <bool FLUX> struct WsCfg {
  static constexpr int PROD = FLUX ? 64 : 256;           // producer threads
  static constexpr int RPT = PROD < TC_M ? TC_M / PROD : 1;  // A rows per producer thread
  static constexpr int SPT = 8 * TC_M / (PROD * RPT);   // samples of a chunk per thread and row
  static constexpr int AHEAD = FLUX ? 1 : 3;             // chunks of samples loaded ahead
  static constexpr int EPI = FLUX ? 512 : 384;           // epilogue threads: EPI / 128 groups of four warps
  static constexpr int NGRP = EPI / 128;
  static constexpr int EAHEAD = FLUX ? 1 : 2;            // accumulator chunks loaded ahead
  static constexpr int THREADS = PROD + EPI + 32;
  static constexpr int MMA_WARP = (PROD + EPI) / 32;
};

struct WsArgs {
  const float2* S;  // the sample ring [nk][P]
  long P;
  int nk;
  const float* Bt;  // B operands of the nk samples (k_twiddle_tc)
  float4* fd;       // double-float accumulators [nof][P]
  int fd_zero;      // they hold no sum yet: taken as zeros, not read
  int nof, ngroups;
  long nitems;      // row tiles x frequency groups
  // flux mode
  const FluxFace* faces;
  FluxTiles ft;
  double* part;
  int* err;
};

__device__ __forceinline__ void mbar_expect_tx_only(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.expect_tx.relaxed.cta.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

template <bool FLUX> struct WsRow {
  long p0;  // commit: first point of the tile
  int np;   // commit: points of the tile
  FluxFace F;
  long L0;
  int nl, tile;
};

template <bool FLUX> __device__ __forceinline__ WsRow<FLUX> ws_item(const WsArgs& A, long item, int& g) {
  WsRow<FLUX> r{};
  g = (int)(item % A.ngroups);
  const long t = item / A.ngroups;
  r.tile = (int)t;
  if (FLUX) {
    int f = 0, fs = 0;
#pragma unroll
    for (int i = 1; i < 6; ++i)
      if (t >= A.ft.start[i]) {
        f = i;
        fs = A.ft.start[i];
      }
    r.F = A.faces[f];
    r.L0 = (t - fs) * FL_LOC;
    r.nl = (int)min((long)FL_LOC, r.F.n - r.L0);
  } else {
    r.p0 = t * TC_M;
    r.np = (int)min((long)TC_M, A.P - r.p0);
  }
  return r;
}

// Sample point of A row `row` (-1: none).
template <bool FLUX> __device__ __forceinline__ long ws_point(const WsRow<FLUX>& r, int row) {
  if (FLUX) {
    const int c = row & 3, l = ((row >> 5) << 3) + ((row & 31) >> 2);
    return l < r.nl ? face_comp(r.F, c) + r.L0 + l : -1;
  }
  return row < r.np ? r.p0 + row : -1;
}

template <bool FLUX> __device__ __forceinline__ void dft_ws(const WsArgs& A) {
  constexpr int WS_PROD = WsCfg<FLUX>::PROD, RPT = WsCfg<FLUX>::RPT, WS_MMA_WARP = WsCfg<FLUX>::MMA_WARP;
  constexpr int WS_EPI = WsCfg<FLUX>::EPI, NG = WsCfg<FLUX>::NGRP, EA = WsCfg<FLUX>::EAHEAD;
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ uint64_t full[WS_STAGES], empty[WS_STAGES], accf[2], acce[2], fin;
  __shared__ uint32_t taddr_s;
  __shared__ int stop_s;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int code = FLUX ? 5 : 3;
  const int nch = (2 * A.nk + TC_KC - 1) / TC_KC;
  const long per = (long)TC_BROWS * TC_KC;
  const bool mma = A.nk > 0;
  if (tid == 0) {
    for (int s = 0; s < WS_STAGES; ++s) {
      mbar_init(&full[s], WS_PROD);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&accf[b], 1);
      mbar_init(&acce[b], WS_EPI);
    }
    mbar_init(&fin, 1);
    stop_s = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == WS_MMA_WARP && mma) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&taddr_s)),
                 "r"(2 * TC_NMAX)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = mma ? taddr_s : 0u;
  auto give_up = [&]() {
    atomicExch(A.err, code);
    *(volatile int*)&stop_s = 1;
  };
  auto stopped = [&]() { return *(volatile int*)&stop_s != 0; };

  if (tid < WS_PROD) {
    // ---- producers: one flat sequence of (item, chunk) pairs; a thread takes
    // RPT rows (row0 + h WS_PROD) and SPT of a chunk's 8 samples from q0, the
    // samples of the next AHEAD chunks in registers while a chunk is split
    // into its stage
    if (mma) {
      constexpr int SPT = WsCfg<FLUX>::SPT, AH = WsCfg<FLUX>::AHEAD;
      const int row0 = tid % TC_M, q0 = (tid / TC_M) * SPT;
      int armed[WS_STAGES] = {};  // fills issued per stage (thread 0: the last one is drained at exit)
      struct Cur {
        long j;
        int c, g;
        long rp[RPT];
        bool ok;
      };
      auto at = [&](long j, int c) {
        Cur x;
        x.j = j;
        x.c = c;
        x.g = 0;
        x.ok = false;
#pragma unroll
        for (int h = 0; h < RPT; ++h) x.rp[h] = -1;
        const long item = blockIdx.x + j * gridDim.x;
        if (item < A.nitems) {
          const WsRow<FLUX> r = ws_item<FLUX>(A, item, x.g);
#pragma unroll
          for (int h = 0; h < RPT; ++h) {
            x.rp[h] = ws_point<FLUX>(r, row0 + h * WS_PROD);
            if (!bc_ok(x.rp[h] < A.P, BC_DFT_SAMPLE, x.rp[h])) x.rp[h] = -1;
          }
          x.ok = true;
        }
        return x;
      };
      auto next = [&](const Cur& x) {
        if (x.c + 1 < nch) {
          Cur y = x;
          ++y.c;
          return y;
        }
        return at(x.j + 1, 0);
      };
      constexpr int NV = SPT * RPT;  // samples a thread holds per chunk
      auto load = [&](const Cur& x, float2* dst) {
#pragma unroll
        for (int q = 0; q < SPT; ++q) {
          const int k = x.c * (TC_KC / 2) + q0 + q;
          const bool kk = x.ok && k < A.nk;
#pragma unroll
          for (int h = 0; h < RPT; ++h)
            dst[SPT * h + q] = (kk && x.rp[h] >= 0) ? A.S[(long)k * A.P + x.rp[h]] : make_float2(0.f, 0.f);
        }
      };
      // a register ring of AHEAD + 1 chunks: v[0] is split while v[1..AHEAD]
      // are in flight (constant indices after unrolling)
      Cur cu[AH + 1];
      float2 v[AH + 1][NV];
      cu[0] = at(0, 0);
#pragma unroll
      for (int d = 1; d <= AH; ++d) cu[d] = next(cu[d - 1]);
#pragma unroll
      for (int d = 0; d < AH; ++d) load(cu[d], v[d]);
      for (long n = 0; cu[0].ok && !stopped(); ++n) {
        load(cu[AH], v[AH]);
        const int s = (int)(n % WS_STAGES);
        const long u = n / WS_STAGES;
        if (u > 0 && !mbar_wait(&empty[s], (unsigned)((u - 1) & 1), STREAM_WAIT_CYCLES)) {
          give_up();
          break;
        }
        unsigned char* st = smem + s * TC_STAGE;
        if (tid == 0) {
          const int ncol = ((2 * min(TC_NW, A.nof - cu[0].g * TC_NW) + 15) / 16) * 16;
          const unsigned nb = (unsigned)(ncol * TC_KC * 4);
          const float* src = A.Bt + ((long)(cu[0].g * nch + cu[0].c) * 2) * per;
          mbar_expect_tx_only(&full[s], 2 * nb);
          fence_proxy_async();
          bulk_g2s(st + 2 * TC_A_BYTES, src, nb, &full[s]);
          bulk_g2s(st + 2 * TC_A_BYTES + TC_B_BYTES, src + per, nb, &full[s]);
          ++armed[s];
        }
        float* Ah = (float*)st;
        float* Al = (float*)(st + TC_A_BYTES);
#pragma unroll
        for (int h = 0; h < RPT; ++h) {
          const int row = row0 + h * WS_PROD;
#pragma unroll
          for (int m = 0; m < SPT / 2; ++m) {
            const float2 a = v[0][SPT * h + 2 * m], bq = v[0][SPT * h + 2 * m + 1];
            const float4 x = make_float4(a.x, a.y, bq.x, bq.y);
            const float4 hv = make_float4(tf32_hi(x.x), tf32_hi(x.y), tf32_hi(x.z), tf32_hi(x.w));
            const int col = 2 * q0 + 4 * m;  // K column of sample q0 + 2 m
            *(float4*)(Ah + tc_off(row, col)) = hv;
            *(float4*)(Al + tc_off(row, col)) = make_float4(x.x - hv.x, x.y - hv.y, x.z - hv.z, x.w - hv.w);
          }
        }
        fence_proxy_async();  // the generic-proxy writes of A before the tensor core reads them
        mbar_arrive(&full[s]);
#pragma unroll
        for (int d = 0; d < AH; ++d) {
#pragma unroll
          for (int q = 0; q < NV; ++q) v[d][q] = v[d + 1][q];
          cu[d] = cu[d + 1];
        }
        cu[AH] = next(cu[AH - 1]);
      }
      if (tid == 0)
        // copies issued into a stage whose MMAs never ran must land before the CTA exits
        for (int s = 0; s < WS_STAGES; ++s)
          if (armed[s] && stopped()) mbar_wait(&full[s], (unsigned)((armed[s] - 1) & 1), STREAM_WAIT_CYCLES);
    }
  } else if (warp == WS_MMA_WARP) {
    // ---- the MMA thread
    if (mma && lane == 0) {
      long n = 0, j = 0;
      for (long item = blockIdx.x; item < A.nitems && !stopped(); item += gridDim.x, ++j) {
        const int b = (int)(j & 1);
        const long vv = j >> 1;
        if (j >= 2 && !mbar_wait(&acce[b], (unsigned)((vv - 1) & 1), STREAM_WAIT_CYCLES)) {
          give_up();
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const int g = (int)(item % A.ngroups);
        const int ncol = ((2 * min(TC_NW, A.nof - g * TC_NW) + 15) / 16) * 16;
        const uint32_t idesc = tc_idesc(ncol), acc = tmem + (uint32_t)(b * TC_NMAX);
        bool ok = true;
        for (int c = 0; c < nch; ++c, ++n) {
          const int s = (int)(n % WS_STAGES);
          const long u = n / WS_STAGES;
          if (!mbar_wait(&full[s], (unsigned)(u & 1), STREAM_WAIT_CYCLES)) {
            ok = false;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          unsigned char* st = smem + s * TC_STAGE;
          const float* Ah = (const float*)st;
          const float* Al = (const float*)(st + TC_A_BYTES);
          const float* Bh = (const float*)(st + 2 * TC_A_BYTES);
          const float* Bl = (const float*)(st + 2 * TC_A_BYTES + TC_B_BYTES);
#pragma unroll
          for (int ks = 0; ks < TC_KC / 8; ++ks) {
            const uint64_t ah = tc_desc(Ah + 64 * ks), al = tc_desc(Al + 64 * ks);
            const uint64_t bh = tc_desc(Bh + 64 * ks), bl = tc_desc(Bl + 64 * ks);
            tc_mma(acc, ah, bh, idesc, (c > 0 || ks > 0) ? 1 : 0);
            tc_mma(acc, ah, bl, idesc, 1);
            tc_mma(acc, al, bh, idesc, 1);
          }
          tc_commit(&empty[s]);
        }
        if (!ok) {
          give_up();
          break;
        }
        tc_commit(&accf[b]);
      }
      // every MMA issued has completed before the TMEM is freed
      tc_commit(&fin);
      mbar_wait(&fin, 0, STREAM_WAIT_CYCLES);
    }
  } else {
    // ---- epilogue: warp w reads TMEM lanes 32 (w % 4); group (w - PROD/32) / 4
    // takes the 4-frequency chunks of its index mod NG
    const int q4 = warp & 3, grp = (warp - WS_PROD / 32) >> 2;
    long j = 0;
    for (long item = blockIdx.x; item < A.nitems; item += gridDim.x, ++j) {
      if (__any_sync(0xffffffffu, stopped())) break;
      const int b = (int)(j & 1);
      const long vv = j >> 1;
      int g;
      const WsRow<FLUX> r = ws_item<FLUX>(A, item, g);
      long ep = ws_point<FLUX>(r, 32 * q4 + lane);
      if (!bc_ok(ep < A.P, BC_DFT_POINT, ep)) ep = -1;
      const int nw = min(TC_NW, A.nof - g * TC_NW), nchk = (nw + WS_FCH - 1) / WS_FCH;
      float4* fdg = A.fd + (long)g * TC_NW * A.P;
      auto load_fd = [&](int ch, float4* dst) {
#pragma unroll
        for (int q = 0; q < WS_FCH; ++q)
          dst[q] = (ep >= 0 && !A.fd_zero && WS_FCH * ch + q < nw) ? fdg[(long)(WS_FCH * ch + q) * A.P + ep]
                                                                   : make_float4(0.f, 0.f, 0.f, 0.f);
      };
      float4 fa[WS_FCH], fb[WS_FCH], fc[EA > 1 ? WS_FCH : 1];
      if (grp < nchk) load_fd(grp, fa);
      if (EA > 1 && grp + NG < nchk) load_fd(grp + NG, fb);
      if (mma) {
        const bool ok = __all_sync(0xffffffffu, mbar_wait(&accf[b], (unsigned)(vv & 1), STREAM_WAIT_CYCLES));
        if (!ok) {
          if (lane == 0) give_up();
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      }
      for (int ch = grp; ch < nchk; ch += NG) {
        if constexpr (EA > 1) {
          if (ch + 2 * NG < nchk) load_fd(ch + 2 * NG, fc);
        } else {
          if (ch + NG < nchk) load_fd(ch + NG, fb);
        }
        if (mma) {
          uint32_t t[2 * WS_FCH];
          const uint32_t ta = tmem + ((uint32_t)(32 * q4) << 16) + (uint32_t)(b * TC_NMAX + 2 * WS_FCH * ch);
          asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];\n"
                       : "=r"(t[0]), "=r"(t[1]), "=r"(t[2]), "=r"(t[3]), "=r"(t[4]), "=r"(t[5]), "=r"(t[6]), "=r"(t[7])
                       : "r"(ta)
                       : "memory");
          asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
          for (int q = 0; q < WS_FCH; ++q) {
            if (FLUX) {
              fa[q].x = df_add_hi(fa[q].x, fa[q].z, __uint_as_float(t[2 * q]));
              fa[q].y = df_add_hi(fa[q].y, fa[q].w, __uint_as_float(t[2 * q + 1]));
            } else {
              acc_add(fa[q], __uint_as_float(t[2 * q]), __uint_as_float(t[2 * q + 1]));
            }
          }
        }
        if (FLUX) {
          // lane 4 l + c holds component c of location 8 q4 + l.  Per
          // frequency the values are scaled by a power of two that brings the
          // warp's largest to [1, 2) (undone exactly when the sum is widened),
          // so that fields far below 1 (the pulse's leading tail) neither
          // underflow nor lose precision in FP32 products; values far below
          // the warp's largest do not count.  Lanes c = 0 and c = 2 form
          // Re(a conj b) and -Re(c conj d) with their partner lane (c ^ 1);
          // the four frequencies' 32 lane values are then summed in one
          // transposed butterfly (fixed order): lane 8 q + 0 ends with the
          // sum of frequency q, which goes out in FP64.
          float v[WS_FCH];
          int sc[WS_FCH];
#pragma unroll
          for (int q = 0; q < WS_FCH; ++q) {
            // the larger magnitude (non-negative floats order as their bits)
            const unsigned mb = __float_as_uint(fmaxf(fabsf(fa[q].x), fabsf(fa[q].y)));
            sc[q] = min(126, max(-126, 127 - (int)(__reduce_max_sync(0xffffffffu, mb) >> 23)));
            const float f = __uint_as_float((unsigned)(127 + sc[q]) << 23);
            const float ax = fa[q].x * f, ay = fa[q].y * f;
            const float bx = __shfl_xor_sync(0xffffffffu, ax, 1), by = __shfl_xor_sync(0xffffffffu, ay, 1);
            const float pr = __fmaf_rn(ay, by, __fmul_rn(ax, bx));
            v[q] = (lane & 1) ? 0.f : (lane & 2) ? -pr : pr;
          }
          const bool h16 = (lane & 16) != 0, h8 = (lane & 8) != 0;
          const float w0 = (h16 ? v[2] : v[0]) + __shfl_xor_sync(0xffffffffu, h16 ? v[0] : v[2], 16);
          const float w1 = (h16 ? v[3] : v[1]) + __shfl_xor_sync(0xffffffffu, h16 ? v[1] : v[3], 16);
          float t = (h8 ? w1 : w0) + __shfl_xor_sync(0xffffffffu, h8 ? w0 : w1, 8);
          t += __shfl_xor_sync(0xffffffffu, t, 4);
          t += __shfl_xor_sync(0xffffffffu, t, 2);
          t += __shfl_xor_sync(0xffffffffu, t, 1);
          const int qq = lane >> 3;
          const int myc = qq == 0 ? sc[0] : qq == 1 ? sc[1] : qq == 2 ? sc[2] : sc[3];
          if ((lane & 7) == 0 && WS_FCH * ch + qq < nw)
            A.part[(long)(g * TC_NW + WS_FCH * ch + qq) * (4L * A.ft.start[6]) + 4L * r.tile + q4] =
                scaled_double(t, -2 * myc);
        } else if (ep >= 0) {
#pragma unroll
          for (int q = 0; q < WS_FCH; ++q)
            if (WS_FCH * ch + q < nw) fdg[(long)(WS_FCH * ch + q) * A.P + ep] = fa[q];
        }
#pragma unroll
        for (int q = 0; q < WS_FCH; ++q) fa[q] = fb[q];
        if constexpr (EA > 1) {
#pragma unroll
          for (int q = 0; q < WS_FCH; ++q) fb[q] = fc[q];
        }
      }
      if (mma) {
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        mbar_arrive(&acce[b]);
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == WS_MMA_WARP && mma)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * TC_NMAX) : "memory");
}

__global__ void __maxnreg__(80) k_dft_ws_commit(WsArgs A) { dft_ws<false>(A); }
__global__ void __launch_bounds__(WsCfg<true>::THREADS, 1) k_dft_ws_flux(WsArgs A) { dft_ws<true>(A); }

// J[f][iw] = scale * sign * (sum of face f's partials, four per tile, in
// order within each thread, then a fixed tree).
__global__ void __launch_bounds__(256) k_flux_sum(const double* __restrict__ part, FluxTiles ft,
                                                  const FluxFace* __restrict__ faces, int nof, double scale,
                                                  double* __restrict__ J) {
  __shared__ double red[256];
  const int iw = blockIdx.x, f = blockIdx.y;
  const long nparts = 4L * ft.start[6];  // one partial per tile and TMEM lane quarter
  long t0 = 0, t1 = 0;
#pragma unroll
  for (int i = 0; i < 6; ++i)
    if (i == f) {
      t0 = 4L * ft.start[i];
      t1 = 4L * ft.start[i + 1];
    }
  double s = 0.0;
  for (long t = t0 + threadIdx.x; t < t1; t += blockDim.x) s += part[(long)iw * nparts + t];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) J[f * nof + iw] = scale * (faces[f].sign > 0 ? red[0] : -red[0]);
}

// Tiles of FL_LOC locations per face of one set of six flux faces.
FluxTiles flux_tiles(const FluxFace* f6) {
  FluxTiles ft{};
  for (int f = 0; f < 6; ++f)
    ft.start[f + 1] = ft.start[f] + (f6[f].active ? (int)((f6[f].n + FL_LOC - 1) / FL_LOC) : 0);
  return ft;
}

// ---------------------------------------------------------------------------
// Persistent whole-step kernel for small grids (IRIS_STENCIL_PERSISTENT).
//
// On a grid of a few thousand cells each operator launch of a step costs a
// few microseconds of launch latency for well under a microsecond of work.
// k_tiny runs a span of steps in one cooperative launch (every CTA resident
// at once): per step the E pass, the H pass, the TF/SF corrections and the
// DFT sample, each a grid-stride loop over its work with the split passes'
// per-cell functions, separated by grid-wide barriers.  The arithmetic and
// every value stored are the split passes', so the results are theirs bit
// for bit.  What shapes it is GB300's FP64 rate (two FP64 instructions a
// cycle per SM, one warp instruction every 64 cycles on a sub-partition):
//   * a pass costs its busiest sub-partition's FP64 instruction count, so
//     in FP64 every cell is split over three work items, one per component
//     (the Bloch ghost products of a cell on the x or y border cost as much
//     as its update), component-major so that a warp's items take one path,
//     spread over every SM, the UPML items on threads that do no second
//     item; cells outside the UPML slabs run code compiled without the slab
//     branch.  FP64 rounds every operation explicitly, so
//     any split gives the split passes' values; FP32 arithmetic may be
//     contracted to FMAs differently in a different instantiation, so FP32
//     keeps the split passes' own per-cell function, one item per cell;
//   * the TF/SF corrections' incident field (exp, sincos and divisions in
//     FP64, a dependent chain of a few hundred FP64 instructions) is
//     evaluated for every step of the span up front by k_tfsf_table, in
//     parallel; the TF/SF phase only adds the tabulated values, one thread
//     per corrected row;
//   * the DFT sample reads a flat table of its points' field and storage
//     index (one dependent load, not a walk over the run list), and shares
//     the TF/SF phase (one barrier less a step) when no sample point lies on
//     a plane the corrections write.
// The barrier is an arrival counter in global memory; every wait is bounded
// (about a second): a CTA that gives up records it (code 6) and returns, and
// so do the others at their next wait.

struct GridBar {
  unsigned count;
};

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void red_add_release(unsigned* p, unsigned x) {
  asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(x) : "memory");
}

// All CTAs of the launch reach this point before any passes it; false when
// the wait gave up.  The count only grows within a launch (it is zeroed
// before each): every CTA's thread 0 adds its arrival with release semantics
// and waits, with acquire loads, until the count reaches its target, nblk
// per barrier passed so far (thread 0's copy of target is the one used).
// One arrival without a returned value and one load per poll: measured on
// GB300 at 1.1-1.2 microseconds a barrier for 72 or 152 CTAs, against 1.7
// for an arrival counter reset by the last arriver plus a generation word.
__device__ __forceinline__ bool grid_barrier(GridBar* b, unsigned& target, unsigned nblk, int* err,
                                             long long limit = STREAM_WAIT_CYCLES) {
  __shared__ int ok_s;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    target += nblk;
    red_add_release(&b->count, 1u);
    const long long t0 = clock64();
    while ((int)(ld_acquire_u32(&b->count) - target) < 0)
      if (clock64() - t0 > limit) {
        ok = 0;
        break;
      }
    if (!ok) atomicExch(err, 6);
    ok_s = ok;
  }
  __syncthreads();
  return ok_s != 0;
}

template <typename T> struct TinyArgs {
  FieldArgs<T> a;
  SrcArgs s;
  const TfsfVal* tfv;    // TF/SF corrections per [step of the span][ix in 0..nx+1]
  int merged;            // the DFT sample runs in the TF/SF phase
  const long* sidx;      // per sample point: storage index * 8 + field (0..5)
  const Seg* segs;
  int nsegs;
  typename V2<T>::t* S;  // the DFT ring
  long P;
  int* tk;
  int slot0;             // first free ring slot
  int it0, n;            // steps it0 .. it0 + n - 1
  int to_fourier, sample_fourier, dft;
  GridBar* bar;
  int* err;
};

// Threads per CTA: 128 while the work items (three a cell in FP64, one in
// FP32) spread that thinly over the SMs, up to 1024 as the grid grows (the
// kernel is compiled for 1024, so at most 64 registers a thread).
constexpr int TINY_MIN_THREADS = 128, TINY_MAX_THREADS = 1024;

// IRIS_OP_BARRIER_CHECK: a cooperative launch of two CTAs in which the second
// returns without arriving, so the first waits at the grid barrier with the
// persistent kernel's limit divided by 2^shift, gives up and records it.
__global__ void k_barrier_check(GridBar* bar, int* err, int shift) {
  unsigned target = 0;
  if (blockIdx.x != 0) return;
  grid_barrier(bar, target, 2, err, STREAM_WAIT_CYCLES >> shift);
}

// The TF/SF corrections of steps it0 .. it0+n-1 for every column ix in
// [0, nx+1] (tfsf_values, the split passes' function).
__global__ void k_tfsf_table(SrcArgs s, int it0, int n, int ncol, TfsfVal* __restrict__ out) {
  const long j = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= (long)n * ncol) return;
  cx<double> vE, vH;
  tfsf_values(s, it0 + (int)(j / ncol), (int)(j % ncol), vE, vH);
  out[j] = TfsfVal{vE.re, vE.im, vH.re, vH.im};
}

// FP64 work items of k_tiny: component k of a cell, UPML cells with the slab
// code, the others without.  The grid-stride loop gives the threads below
// nitems - stride two items; the UPML items (about 1.5 times an interior
// item's FP64 work) go to the positions of one-item threads, so that no
// thread does a UPML item and a second one.  Position w maps to UPML item
// w - u0 in [u0, u0 + nu3) and to interior item w (w < u0) or w - nu3.
struct TinyMap {
  int lo, hi0;         // UPML planes 1..lo and hi0..nz
  unsigned nxy, nuc, nic;  // cells per plane, UPML cells, interior cells
  unsigned u0;             // first position of the UPML items
  __device__ __forceinline__ void item(unsigned w, int nx, int& k, int& x, int& y, int& z, bool& upml) const {
    unsigned c;
    upml = w >= u0 && w < u0 + 3 * nuc;
    if (upml) {
      const unsigned u = w - u0;
      k = (int)(u / nuc);
      c = u - (unsigned)k * nuc;
      const unsigned pl = c / nxy;
      z = pl < (unsigned)lo ? (int)pl + 1 : hi0 + (int)(pl - lo);
    } else {
      const unsigned v = w < u0 ? w : w - 3 * nuc;
      k = (int)(v / nic);
      c = v - (unsigned)k * nic;
      z = lo + 1 + (int)(c / nxy);
    }
    const unsigned r = c % nxy;
    x = (int)(r % (unsigned)nx) + 1;
    y = (int)(r / (unsigned)nx) + 1;
  }
};
template <bool CEPS, int MASK>
__device__ __forceinline__ void tiny_e(const FieldArgs<double>& a, int x, int y, int z, bool upml) {
  if (upml) e_split_cell<double, CEPS, true, MASK>(a, x, y, z);
  else e_split_cell<double, CEPS, false, MASK>(a, x, y, z);
}
template <int MASK> __device__ __forceinline__ void tiny_h(const FieldArgs<double>& a, int x, int y, int z, bool upml) {
  if (upml) h_split_cell<double, true, MASK>(a, x, y, z);
  else h_split_cell<double, false, MASK>(a, x, y, z);
}

template <typename T, bool CEPS> __global__ void __launch_bounds__(TINY_MAX_THREADS) k_tiny(TinyArgs<T> A) {
  using V = typename V2<T>::t;
  const Geo g = A.a.g;
  const long nxy = (long)g.nx * g.ny, ncell = nxy * g.nz;
  const long gt = (long)blockIdx.x * blockDim.x + threadIdx.x, gs = (long)gridDim.x * blockDim.x;
  const long tf_rows = (long)(g.nx + 2) * (g.ny + 2);
  constexpr bool SPLIT = std::is_same<T, double>::value;
  const long nitems = SPLIT ? 3 * ncell : ncell;
  TinyMap tm;
  tm.lo = min(max(A.a.pmlzi, 0), g.nz);
  tm.hi0 = max(A.a.pmlzf, tm.lo + 1);
  tm.nxy = (unsigned)nxy;
  tm.nuc = (unsigned)(nxy * (tm.lo + max(0, g.nz - tm.hi0 + 1)));
  tm.nic = (unsigned)ncell - tm.nuc;
  tm.u0 = (unsigned)min(max(nitems - gs, 0L), nitems - 3L * tm.nuc);
  unsigned target = 0;  // grid barrier target
  int slot = A.slot0;
  for (int i = 0; i < A.n; ++i) {
    const int it = A.it0 + i;
    for (long w = gt; w < nitems; w += gs) {
      // 32-bit index arithmetic: the host keeps 3 x cells below 2^31
      if constexpr (SPLIT) {
        int k, x, y, z;
        bool upml;
        tm.item((unsigned)w, g.nx, k, x, y, z, upml);
        if (k == 0) tiny_e<CEPS, 1>(A.a, x, y, z, upml);
        else if (k == 1) tiny_e<CEPS, 2>(A.a, x, y, z, upml);
        else tiny_e<CEPS, 4>(A.a, x, y, z, upml);
      } else {
        const unsigned r = (unsigned)w % (unsigned)nxy;
        e_split_cell<T, CEPS>(A.a, (int)(r % (unsigned)g.nx) + 1, (int)(r / (unsigned)g.nx) + 1,
                              (int)((unsigned)w / (unsigned)nxy) + 1);
      }
    }
    if (!grid_barrier(A.bar, target, gridDim.x, A.err)) return;
    for (long w = gt; w < nitems; w += gs) {
      // 32-bit index arithmetic: the host keeps 3 x cells below 2^31
      if constexpr (SPLIT) {
        int k, x, y, z;
        bool upml;
        tm.item((unsigned)w, g.nx, k, x, y, z, upml);
        if (k == 0) tiny_h<1>(A.a, x, y, z, upml);
        else if (k == 1) tiny_h<2>(A.a, x, y, z, upml);
        else tiny_h<4>(A.a, x, y, z, upml);
      } else {
        const unsigned r = (unsigned)w % (unsigned)nxy;
        h_split_cell<T>(A.a, (int)(r % (unsigned)g.nx) + 1, (int)(r / (unsigned)g.nx) + 1,
                        (int)((unsigned)w / (unsigned)nxy) + 1);
      }
    }
    if (!grid_barrier(A.bar, target, gridDim.x, A.err)) return;
    const bool sample = A.dft && it >= A.to_fourier && it % A.sample_fourier == 0;
    const bool tf = A.s.variant != 0;
    // TF/SF rows (one thread per (ix, iy) of the ranges k_tfsf covers), then
    // the sample points; in one phase when merged, else separated by a barrier
    const long n_tf = tf ? tf_rows : 0, n_s = sample ? A.P : 0;
    const bool one = sample && A.merged;
    for (long w = gt; w < (one ? n_tf + n_s : n_tf); w += gs) {
      if (w < n_tf) {
        const int ix = (int)(w % (g.nx + 2)), iy = (int)(w / (g.nx + 2));
        const TfsfVal v = A.tfv[(long)i * (g.nx + 2) + ix];
        tfsf_apply<T>(A.a.e, A.a.h, g, A.s, ix, iy, iy, cx<double>{v.er, v.ei}, cx<double>{v.hr, v.hi});
      } else {
        const long q = w - n_tf, code = A.sidx[q];
        const int f = (int)(code & 7);
        if (bc_ok(f < 6 && (code >> 3) < g.comp, BC_GATHER_SRC, code >> 3))
          A.S[(long)slot * A.P + q] = (f < 3 ? A.a.e + f * g.comp : A.a.h + (f - 3) * g.comp)[code >> 3];
      }
    }
    if (tf && !one && !grid_barrier(A.bar, target, gridDim.x, A.err)) return;
    if (sample) {
      if (!one)
        for (long q = gt; q < A.P; q += gs) {
          const long code = A.sidx[q];
          const int f = (int)(code & 7);
          if (bc_ok(f < 6 && (code >> 3) < g.comp, BC_GATHER_SRC, code >> 3))
            A.S[(long)slot * A.P + q] = (f < 3 ? A.a.e + f * g.comp : A.a.h + (f - 3) * g.comp)[code >> 3];
        }
      if (gt == 0) A.tk[slot] = it + 1 - A.to_fourier;
      ++slot;
      // the next step's E pass overwrites what was just sampled
      if (!grid_barrier(A.bar, target, gridDim.x, A.err)) return;
    }
  }
}

// ---------------------------------------------------------------------------
// Material generators: the structure's eps_inv over planes hi..hf (ghost
// rows and columns included) built on the device, the voxelisers of the
// geometry front-end (slit() of code/mesh.f90:57-69 generalised), value for
// value what the host voxelisers compute:
//   kind 1 (spheres): 1/eps_bbox, then for each sphere (cx, cy, cz, r, eps)
//     in order, 1/eps where ((z-cz)^2 + (y-cy)^2) + (x-cx)^2 <= r^2 over the
//     sphere's bounding box (z clipped to [hi, hf], x and y at most nx and
//     ny cells from floor(c - r), taken modulo the period); later spheres
//     win;
//   kind 2 (pattern): 1/eps_in where the i-th SplitMix64 draw of the seed is
//     below fill, else 1/eps_out, i = ((z-hi) ny + y-1) nx + x-1;
//   kind 3 (design region): 1/(emin + (emax-emin) u_i) over [x0,x1] x [y0,y1],
//     i in the region's own (z, y, x) order, 1/eps_bbox elsewhere.
// Kinds 1 and 2 fill the ghost rows and columns with their periodic images;
// kind 3 leaves them at 1/eps_bbox.  FP64 operations are the host's, one
// rounding each.
// A sphere as the generator reads it: centre, r^2 and 1/eps, and its
// bounding box, the z planes [zlo, zhi] and the x and y ranges xlo .. xlo +
// lx - 1, ylo .. ylo + ly - 1 (periodic in x and y); built on the host, with
// the same IEEE operations, once per sphere rather than once per cell.
struct SphereBox {
  double cx, cy, cz, r2, inv;
  int zlo, zhi, xlo, lx, ylo, ly;
};

// Spheres binned per (plane, 32 x 32 tile of x, y): lst[off[b] .. off[b+1])
// holds, ascending, the spheres whose bounding box touches bin b = ((z - hi)
// nty + ty) ntx + tx; null when the lists would be too long (the generator
// then tests every sphere).
constexpr int GEN_TILE = 32;

struct GenArgs {
  int kind, hi, hf;
  double base;
  const SphereBox* sph;
  int nsph;
  const int* off;
  const int* lst;
  int ntx, nty;
  unsigned long long seed;
  double fill, v_in, v_out;
  int x0, x1, y0, y1;
  double emin, emax;
};

__device__ __forceinline__ double splitmix_u(unsigned long long seed, unsigned long long i) {
  unsigned long long z = seed + (i + 1ull) * 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  return (double)(z >> 11) * (1.0 / 9007199254740992.0);
}

template <typename T> __global__ void k_material_gen(GenArgs G, Geo g, T* __restrict__ out) {
  const long nx2 = g.nx + 2, nxy = nx2 * (g.ny + 2);
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const int nzs = G.hf - G.hi + 1;
  if (t >= nxy * nzs) return;
  const int zz = (int)(t / nxy);
  const long rr = t % nxy;
  const int y = (int)(rr / nx2), x = (int)(rr % nx2), z = G.hi + zz;
  double v = G.base;
  if (G.kind == 3) {
    if (x >= G.x0 && x <= G.x1 && y >= G.y0 && y <= G.y1) {
      const unsigned long long nxr = G.x1 - G.x0 + 1, nyr = G.y1 - G.y0 + 1;
      const unsigned long long i = ((unsigned long long)zz * nyr + (unsigned long long)(y - G.y0)) * nxr + (x - G.x0);
      v = __ddiv_rn(1.0, __dadd_rn(G.emin, __dmul_rn(__dsub_rn(G.emax, G.emin), splitmix_u(G.seed, i))));
    }
  } else {
    const int xs = x == 0 ? g.nx : x == g.nx + 1 ? 1 : x;
    const int ys = y == 0 ? g.ny : y == g.ny + 1 ? 1 : y;
    if (G.kind == 2) {
      const unsigned long long i =
          ((unsigned long long)zz * g.ny + (unsigned long long)(ys - 1)) * (unsigned long long)g.nx + (xs - 1);
      v = splitmix_u(G.seed, i) < G.fill ? G.v_in : G.v_out;
    } else {
      // the last sphere that holds the cell wins: search from the last
      auto inside = [&](const SphereBox& b) {
        if (z < b.zlo || z > b.zhi) return false;
        const int xu = b.xlo + ((xs - b.xlo) % g.nx + g.nx) % g.nx, yu = b.ylo + ((ys - b.ylo) % g.ny + g.ny) % g.ny;
        if (xu > b.xlo + b.lx - 1 || yu > b.ylo + b.ly - 1) return false;
        const double dz = __dsub_rn((double)z, b.cz), dy = __dsub_rn((double)yu, b.cy), dx = __dsub_rn((double)xu, b.cx);
        const double d2 = __dadd_rn(__dadd_rn(__dmul_rn(dz, dz), __dmul_rn(dy, dy)), __dmul_rn(dx, dx));
        return d2 <= b.r2;
      };
      if (G.off) {
        const long bin = ((long)zz * G.nty + (ys - 1) / GEN_TILE) * G.ntx + (xs - 1) / GEN_TILE;
        for (int j = G.off[bin + 1] - 1; j >= G.off[bin]; --j) {
          const SphereBox& b = G.sph[G.lst[j]];
          if (inside(b)) {
            v = b.inv;
            break;
          }
        }
      } else {
        for (int k = G.nsph - 1; k >= 0; --k)
          if (inside(G.sph[k])) {
            v = G.sph[k].inv;
            break;
          }
      }
    }
  }
  out[(long)zz * g.plane + (long)y * g.pitch + (x + g.xo)] = (T)v;
}

// Stored material planes hi..hf out to the host (real and imaginary parts).
template <typename T> __global__ void k_material_get(const void* __restrict__ eps, bool cplx, Geo g, int nzs,
                                                     double* __restrict__ re, double* __restrict__ im) {
  const long nx2 = g.nx + 2, nxy = nx2 * (g.ny + 2);
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nxy * nzs) return;
  const long src = (t / nxy) * g.plane + ((t % nxy) / nx2) * g.pitch + (t % nx2) + g.xo;
  if (cplx) {
    const typename V2<T>::t v = ((const typename V2<T>::t*)eps)[src];
    re[t] = (double)v.x;
    im[t] = (double)v.y;
  } else {
    re[t] = (double)((const T*)eps)[src];
    im[t] = 0.0;
  }
}

// ---------------------------------------------------------------------------
// Field transfer in the reference's own layout, complex(8) (3, 0:nx+1,
// 0:ny+1, 0:nz+1) (UPML: (3, 1:nx, 1:ny, planes)), a chunk of z planes at a
// time through a device staging buffer: the host array is read or written
// in place, with no host copy of the field.  Element t of a chunk is
// component t % 3 of location t / 3, x fastest.  pc: component stride of
// the device arrays; ox, oy: the first x and y (0 for fields with ghosts, 1
// for the UPML slabs); at(x, y, z): storage index.
struct XferMap {
  Geo g;       // fields: the engine geometry
  long pc;     // component stride
  int nx, ny;  // extents of x and y in the host layout
  int ox, oy;  // first x, y of the host layout
  int pml;     // 1: UPML slab indexing ((z ny + y-1) nx + x-1)
  __device__ __forceinline__ long at(int x, int y, int z) const {
    return pml ? ((long)z * (ny) + (y - 1)) * (long)nx + (x - 1) : g.at(x, y, z);
  }
};

template <typename T>
__global__ void k_pack(const typename V2<T>::t* __restrict__ f, XferMap m, int z0, long n, double2* __restrict__ out) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int c = (int)(t % 3);
  long r = t / 3;
  const int x = (int)(r % m.nx) + m.ox;
  r /= m.nx;
  const int y = (int)(r % m.ny) + m.oy, z = z0 + (int)(r / m.ny);
  const typename V2<T>::t v = f[c * m.pc + m.at(x, y, z)];
  out[t] = make_double2((double)v.x, (double)v.y);
}

template <typename T>
__global__ void k_unpack(typename V2<T>::t* __restrict__ f, XferMap m, int z0, long n, const double2* __restrict__ in) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int c = (int)(t % 3);
  long r = t / 3;
  const int x = (int)(r % m.nx) + m.ox;
  r /= m.nx;
  const int y = (int)(r % m.ny) + m.oy, z = z0 + (int)(r / m.ny);
  const double2 v = in[t];
  typename V2<T>::t w;
  w.x = (T)v.x;
  w.y = (T)v.y;
  f[c * m.pc + m.at(x, y, z)] = w;
}

// One plane of a field (SDL snapshots): out[(i2 * n1 + i1) * 3 + k].
template <typename T>
__global__ void k_plane(const typename V2<T>::t* __restrict__ f, Geo g, int axis, int index, int lo1, int n1, int lo2,
                        int n2, double2* __restrict__ out) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 3L * n1 * n2) return;
  const int k = (int)(t % 3), i1 = (int)((t / 3) % n1), i2 = (int)(t / (3L * n1));
  const int a = lo1 + i1, b = lo2 + i2;
  const long i = axis == 1 ? g.at(index, a, b) : axis == 2 ? g.at(a, index, b) : g.at(a, b, index);
  const typename V2<T>::t v = f[k * g.comp + i];
  out[t] = make_double2((double)v.x, (double)v.y);
}

// Structure material into the padded layout: planes hi..hf of eps_inv given
// over (hi-1:hf+1, 0:ny+1, 0:nx+1) as re/im (im may be null), or, with
// re == null, the default of set_emconstants and slit() (code/mesh.f90:57-109):
// 1/eps_bbox (vr, vi) with the slit columns aix..afx set to 1.
template <typename T>
__global__ void k_material(const double* __restrict__ re, const double* __restrict__ im, Geo g, int nzs, double vr,
                           double vi, int aix, int afx, T* __restrict__ out_r, typename V2<T>::t* __restrict__ out_c) {
  const long nx2 = g.nx + 2, nxy = nx2 * (g.ny + 2);
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nxy * nzs) return;
  const int zz = (int)(t / nxy);
  const long r = t % nxy;
  const int y = (int)(r / nx2), x = (int)(r % nx2);
  double a = vr, b = vi;
  if (re) {
    a = re[t];
    b = im ? im[t] : 0.0;
  } else if (x >= aix && x <= afx) {
    a = 1.0;
    b = 0.0;
  }
  const long dst = (long)zz * g.plane + (long)y * g.pitch + (x + g.xo);
  if (out_c) {
    typename V2<T>::t v;
    v.x = (T)a;
    v.y = (T)b;
    out_c[dst] = v;
  } else {
    out_r[dst] = (T)a;
  }
}


template <typename ACC>
__global__ void __launch_bounds__(256) k_flux(const ACC* __restrict__ fd, long P, const FluxFace* __restrict__ faces,
                                              int nof, double scale, double* __restrict__ J) {
  __shared__ double red[256];
  const int iw = blockIdx.x, f = blockIdx.y;
  const FluxFace F = faces[f];
  double s = 0.0;
  if (F.active && bc_ok(F.pa >= 0 && F.pb >= 0 && F.pc >= 0 && F.pd >= 0 &&
                            max(max(F.pa, F.pb), max(F.pc, F.pd)) + F.n <= P,
                        BC_FLUX_POINT, F.n)) {
    const ACC* row = fd + (long)iw * P;
    for (long L = threadIdx.x; L < F.n; L += blockDim.x) {
      const double2 a = acc_value(row[F.pa + L]), b = acc_value(row[F.pb + L]), c = acc_value(row[F.pc + L]),
                    d = acc_value(row[F.pd + L]);
      s += (a.x * b.x + a.y * b.y) - (c.x * d.x + c.y * d.y);
    }
  }
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) J[f * nof + iw] = scale * (F.sign > 0 ? red[0] : -red[0]);
}

// ---------------------------------------------------------------------------
// Fused E+H pass (FP32): one CTA per column tile and z chunk of the launch;
// the tile column itself is fused_column (iris_fused.cuh).

template <bool CEPS, bool UPML, typename IT>
__global__ void __launch_bounds__(FZ_X* FZ_Y, 2) k_fused(FusedArgs A) {
  __shared__ FusedSmem S;
  extern __shared__ __align__(16) unsigned char fz_dyn[];
  FusedUpml& U = *reinterpret_cast<FusedUpml*>(fz_dyn);  // UPML = true only
  const bool r0 = (int)blockIdx.z < A.nc0;
  const int z0 = r0 ? A.za0 + A.zc0 * (int)blockIdx.z : A.za1 + A.zc1 * ((int)blockIdx.z - A.nc0);
  const int z1 = min(z0 + (r0 ? A.zc0 : A.zc1) - 1, r0 ? A.zb0 : A.zb1);
  fused_column<CEPS, UPML, IT>(A, S, U, blockIdx.x, blockIdx.y, z0, z1);
}

}  // namespace

// ---------------------------------------------------------------------------
// host side

thread_local std::string g_last_error;

int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}
void clear_error() { g_last_error.clear(); }

}  // namespace iris

using namespace iris;

namespace {

int p2ceil(int n) {
  int v = 1;
  while (v < n) v <<= 1;
  return v;
}

// set_sz(), code/boundary_II.f90:224-276, and the per-plane UPML coefficient
// rows.  Component -> profile permutation of code/boundary_II.f90:86-99:
// D_k decays with profile pd[k]; E_k with profile pe[k].
void make_coef(const iris_params& p, std::vector<double>& rows) {
  const int nb = p.pmlzi, nt = p.nz - p.pmlzf + 1;
  rows.assign((size_t)NCOEF * (nb + nt), 0.0);
  const double dtq2 = (p.dt / p.Q) * (p.dt / p.Q);
  static const int pd[3] = {1, 2, 0}, pe[3] = {2, 0, 1};
  for (int slab = 0; slab < 2; ++slab) {
    const int z0 = slab == 0 ? 1 : p.pmlzf, z1 = slab == 0 ? p.pmlzi : p.nz;
    const double epsb = slab == 0 ? p.eps1 : p.eps3;
    for (int z = z0; z <= z1; ++z) {
      long ip = 1;
      double den = 1.0;
      double sg3, k3;
      if (slab == 0) {
        for (int k = 0; k < p.npml; ++k) { ip *= (long)(p.pmlzi - z); den *= (double)(p.pmlzi - 1); }
        sg3 = std::sqrt(p.eps1) * p.wzpml * ((double)ip / den);
        k3 = 1.0 + std::sqrt(p.eps1) * p.pmlalfa * ((double)ip / den);
      } else {
        for (int k = 0; k < p.npml; ++k) { ip *= (long)(z - p.pmlzf); den *= (double)(p.nz - p.pmlzf); }
        sg3 = std::sqrt(p.eps3) * p.wzpml * (double)ip / den;
        k3 = 1.0 + std::sqrt(p.eps3) * p.pmlalfa * (double)ip / den;
      }
      double fp[3], fm[3];
      for (int c = 0; c < 3; ++c) {
        const double sg = c == 2 ? sg3 : 0.0, kk = c == 2 ? k3 : 1.0;
        fp[c] = 2 * p.eps0 * epsb * kk + p.dt * sg;
        fm[c] = 2 * p.eps0 * epsb * kk - p.dt * sg;
      }
      const int row = slab == 0 ? z - 1 : nb + z - p.pmlzf;
      double* r = rows.data() + (size_t)NCOEF * row;
      for (int k = 0; k < 3; ++k) {
        r[CD_A + k] = fm[pd[k]] / fp[pd[k]];
        r[CD_B + k] = (2 * epsb) / fp[pd[k]];
        r[CE_A + k] = fm[pe[k]] / fp[pe[k]];
        r[CE_B + k] = 1 / (p.eps0 * epsb * fp[pe[k]]);
        r[C_FP + k] = fp[k];
        r[C_FM + k] = fm[k];
        r[CB_B + k] = ((2 * epsb) / fp[pd[k]]) * dtq2;
        r[CH_B + k] = 1 / (p.mu0 * fp[pe[k]]);
      }
    }
  }
}

SrcArgs make_src(const iris_params& p) {
  SrcArgs s{};
  const bool two_d = !(p.ny != 1 && p.nx != 1);
  if (!two_d) s.variant = 1;
  else s.variant = p.i_pol == 2 ? 2 : (p.i_pol == 1 ? 1 : 0);
  if (p.plane_wave != 0 && p.plane_wave != 1) s.variant = 0;  // tfsf_data stays zero
  if (p.i_pol != 1 && p.i_pol != 2) s.variant = 0;
  s.i_pol = p.i_pol;
  s.plane_wave = p.plane_wave;
  s.cosine = p.cosine;
  s.nx = p.nx;
  s.ny = p.ny;
  s.iz_min = p.tfsf_zi;
  s.ixo = p.pmlzi - 50;
  s.izo = p.zopump;
  s.izo_i = p.ratio_angle >= 0 ? (int)((double)p.pmlzi - 3.0 * p.gap) : (int)((double)p.nz + 3.0 * p.gap);
  s.Q = p.Q;
  s.c0dt = p.c0 * p.dt;
  s.ko = 2 * p.pi / (p.wlpump * p.f_abohr);
  s.Dk = p.plane_wave == 1 ? p.gpump * p.Q : p.gap * p.Q;
  double eps_src, sign_kz;
  if (p.tfsf_zi > p.hi) { eps_src = p.eps3; sign_kz = -1.0; }
  else { eps_src = p.eps1; sign_kz = 1.0; }
  s.sign_kz = sign_kz;
  s.eps_src = eps_src;
  s.sq_eps = std::sqrt(eps_src);
  s.sqs = std::sqrt(eps_src) * sign_kz;
  const double DELTA = p.ratio_angle * p.pi / 2.0;
  s.ux = std::cos(DELTA);
  s.uz = std::sin(DELTA);
  s.uzs = s.uz * sign_kz;
  s.amp = p.epump * p.Q;
  s.hcoef = s.amp * (p.dt * p.c0 / p.Q);
  s.eps_in1 = 1.0 / p.eps1;
  const double dtc = p.dt * p.c0 / p.Q;
  s.dtcq2 = (dtc * dtc) * 1.0;  // dtcq2*mu_inv
  s.s1 = std::sqrt(p.eps1);
  s.tincr = p.tincr;
  s.tdecay = p.tdecay;
  return s;
}

int validate(const iris_params& p) {
  auto bad = [](const std::string& m) { return fail(IRIS_EINVAL, m); };
  if (p.nx < 1 || p.ny < 1 || p.nz < 1) return bad("grid sizes must be >= 1");
  if (p.pmlzi < 2) return bad("pmlzi must be >= 2 (set_sz divides by pmlzi-1)");
  if (p.pmlzf > p.nz - 1) return bad("pmlzf must be <= nz-1 (set_sz divides by nz-pmlzf)");
  if (p.pmlzf <= p.pmlzi) return bad("pmlzf must be > pmlzi");
  if (p.hi < 1 || p.hf > p.nz || p.hf < p.hi - 1) return bad("structure range [hi,hf] must lie in [1,nz]");
  if (p.tfsf_zi < 1 || p.tfsf_zi > p.nz) return bad("tfsf_zi must lie in [1,nz]");
  if (p.nof < 1) return bad("nof must be >= 1");
  if (p.sample_fourier < 1) return bad("sample_fourier must be >= 1");
  if (p.npml < 0 || p.npml > 8) return bad("npml out of range");
  if (p.system_model != 0) return bad("system_model must be 0");
  if (p.Q <= 0 || p.dt <= 0) return bad("Q and dt must be > 0");
  if (p.eps1 <= 0 || p.eps3 <= 0) return bad("eps1 and eps3 must be > 0");
  const int* boxes[2] = {p.box1, p.box2};
  const int n[3] = {p.nx, p.ny, p.nz};
  for (int b = 0; b < 2; ++b)
    for (int a = 0; a < 3; ++a) {
      const int lo = boxes[b][2 * a], hi = boxes[b][2 * a + 1];
      if (lo < 1 || hi > n[a] || lo > hi) return bad("DFT box planes must satisfy 1 <= lo <= hi <= n on every axis");
    }
  if (p.precision != IRIS_FP64 && p.precision != IRIS_FP32) return bad("precision must be IRIS_FP64 or IRIS_FP32");
  if (p.stencil < IRIS_STENCIL_DEFAULT || p.stencil > IRIS_STENCIL_PERSISTENT) return bad("unknown stencil variant");
  if (p.stencil == IRIS_STENCIL_FUSED && p.precision != IRIS_FP32) return bad("the fused stencil is FP32 only");
  if (p.stencil == IRIS_STENCIL_STREAM && p.precision != IRIS_FP32) return bad("the streamed stencil is FP32 only");
  if (p.dft_faces != IRIS_DFT_ALL && p.dft_faces != IRIS_DFT_Z) return bad("dft_faces must be IRIS_DFT_ALL or IRIS_DFT_Z");
  if (p.dft_kernel < IRIS_DFT_KERNEL_AUTO || p.dft_kernel > IRIS_DFT_KERNEL_TENSOR) return bad("unknown dft_kernel");
  return IRIS_OK;
}

template <typename T> void launch_e(iris_engine* E) {
  KTimer tm(E, IRIS_KC_E);
  FieldArgs<T> a = field_args<T>(E);
  if constexpr (std::is_same<T, float>::value) {
    if (E->stream && !E->eps_complex) {
      k_stream_e<<<E->sgrd, dim3(SX, SY), STREAM_SMEM_E, E->st>>>(a, E->d_err);
      return;
    }
  }
  if (E->eps_complex) k_update_e<T, true><<<E->grd, E->blk, 0, E->st>>>(a);
  else k_update_e<T, false><<<E->grd, E->blk, 0, E->st>>>(a);
}
template <typename T> void launch_h(iris_engine* E) {
  KTimer tm(E, IRIS_KC_H);
  if constexpr (std::is_same<T, float>::value) {
    if (E->stream && !E->eps_complex) {
      k_stream_h<<<E->sgrd, dim3(SX, SY), STREAM_SMEM_H, E->st>>>(field_args<float>(E), E->d_err);
      return;
    }
  }
  k_update_h<T><<<E->grd, E->blk, 0, E->st>>>(field_args<T>(E));
}
template <typename T> void launch_tfsf(iris_engine* E, int it, const int* itp = nullptr) {
  if (E->src.variant == 0) return;
  KTimer tm(E, IRIS_KC_TFSF);
  using V = typename V2<T>::t;
  k_tfsf<T><<<E->tf_grd, E->tf_blk, 0, E->st>>>((V*)E->e, (V*)E->h, E->g, E->src, it, itp);
}

template <typename T> void dft_sample(iris_engine* E, int t, const int* tp = nullptr) {
  if (E->P == 0) return;
  using V = typename V2<T>::t;
  {
  KTimer tm(E, IRIS_KC_GATHER);
  V* slot = (V*)E->S + (long)E->nslot * E->P;
  dim3 grid((unsigned)((E->max_seg + GATHER_BLOCK - 1) / GATHER_BLOCK), (unsigned)E->segs.size());
  k_dft_gather<T><<<grid, 256, 0, E->st>>>((const V*)E->e, (const V*)E->h, E->g.comp, E->d_segs, slot, E->d_tk,
                                          E->nslot, t, tp, E->P);
  }
  if (++E->nslot == E->K) dft_flush(E);
}

FusedArgs fused_args(const iris_engine* E, int part) {
  FusedArgs a{};
  a.f = field_args<float>(E);
  a.e_new = (float2*)E->e2;
  a.h_new = (float2*)E->h2;
  for (int s = 0; s < 2; ++s) a.d_new[s] = (float2*)E->pml_d2[s];
  const std::vector<int>& r = E->fzr[part];  // (za, zb, zc, n) per range
  a.za0 = r[0], a.zb0 = r[1], a.zc0 = r[2], a.nc0 = r[3];
  a.za1 = r.size() > 4 ? r[4] : 0, a.zb1 = r.size() > 4 ? r[5] : 0, a.zc1 = r.size() > 4 ? r[6] : 1;
  return a;
}

// Share of the fused pass's threads that own a cell of an nx x ny plane
// (each 32 x 16 tile writes 31 x 15 cells).
double fused_fill(int nx, int ny) {
  const long tx = (nx + FZ_OX - 1) / FZ_OX, ty = (ny + FZ_OY - 1) / FZ_OY;
  return (double)nx * ny / ((double)tx * FZ_X * ty * FZ_Y);
}

// z chunks of planes za..zb for a launch over `tiles` column tiles: about
// 32 waves of two CTAs per SM, at least 48 planes each (each chunk also
// reads the H plane below it and forms E' on the plane above it; measured
// on GB300 against 8 waves of at least 16
// planes: 512x512x1024 4.91 against 5.04 ms a pass, 160x160x512 0.378
// against 0.389, 512x512x256 and 256x256x512 the same); appends (za, zb,
// planes per chunk, chunks) to r.
void fused_chunks(std::vector<int>& r, int za, int zb, long tiles) {
  if (zb < za) return;
  const int len = zb - za + 1;
  long nch = std::max(1L, (32L * 152 * 2 + tiles - 1) / tiles);
  nch = std::min<long>(nch, std::max(1, len / 48));
  const int zc = (int)((len + nch - 1) / nch);
  r.insert(r.end(), {za, zb, zc, (len + zc - 1) / zc});
}


// One fused step into the second buffers, swap, then TF/SF and the DFT
// sample on the new state, in the operator order of the split passes; step
// it, or *itp + it when itp is given.
void fused_one(iris_engine* E, int it, const int* itp, bool sampled) {
  {
    // the planes outside the UPML slabs with a kernel without slab code and,
    // concurrently on the second stream, the slabs: the two launches write
    // disjoint planes and read only the old state, so the slab launch fills
    // the SMs the interior launch's last wave leaves idle.  One timer spans
    // the pass.
    const bool both = !E->fzr[0].empty() && !E->fzr[1].empty();
    KTimer tm(E, IRIS_KC_FUSED);
    if (both) {
      cudaEventRecord(E->fz_fork, E->st);
      cudaStreamWaitEvent(E->st2, E->fz_fork, 0);
    }
    for (int part = 0; part < 2; ++part) {
      const std::vector<int>& r = E->fzr[part];
      if (r.empty()) continue;
      const FusedArgs a = fused_args(E, part);
      const dim3 grd(E->fgrd.x, E->fgrd.y, (unsigned)(r[3] + (r.size() > 4 ? r[7] : 0)));
      if (part == 0) {
        if (E->fz_i32) {
          if (E->eps_complex) k_fused<true, false, int><<<grd, E->fblk, 0, E->st>>>(a);
          else k_fused<false, false, int><<<grd, E->fblk, 0, E->st>>>(a);
        } else {
          if (E->eps_complex) k_fused<true, false, long><<<grd, E->fblk, 0, E->st>>>(a);
          else k_fused<false, false, long><<<grd, E->fblk, 0, E->st>>>(a);
        }
      } else {
        cudaStream_t s = both ? E->st2 : E->st;
        if (E->fz_i32) {
          if (E->eps_complex) k_fused<true, true, int><<<grd, E->fblk, FZ_UPML_SMEM, s>>>(a);
          else k_fused<false, true, int><<<grd, E->fblk, FZ_UPML_SMEM, s>>>(a);
        } else {
          if (E->eps_complex) k_fused<true, true, long><<<grd, E->fblk, FZ_UPML_SMEM, s>>>(a);
          else k_fused<false, true, long><<<grd, E->fblk, FZ_UPML_SMEM, s>>>(a);
        }
      }
    }
    if (both) {
      cudaEventRecord(E->fz_join, E->st2);
      cudaStreamWaitEvent(E->st, E->fz_join, 0);
    }
  }
  std::swap(E->e, E->e2);
  std::swap(E->h, E->h2);
  for (int s = 0; s < 2; ++s) std::swap(E->pml_d[s], E->pml_d2[s]);
  launch_tfsf<float>(E, it, itp);
  if (sampled) dft_sample<float>(E, it + 1 - E->p.to_fourier, itp);
}

int step_fused(iris_engine* E, int it0, int n) {
  const iris_params& p = E->p;
  int it = it0;
  while (it < it0 + n) {
    if (graph_ready(E, it, it0 + n - it)) {
      int rc = graph_block(E, it, [&] {
        for (int j = 0; j < E->K; ++j) fused_one(E, j, E->d_it, true);
      });
      if (rc) return rc;
      it += E->K;
      continue;
    }
    fused_one(E, it, nullptr, it >= p.to_fourier && it % p.sample_fourier == 0);
    ++it;
  }
  CK(cudaGetLastError());
  return IRIS_OK;
}

template <typename T> int step_t(iris_engine* E, int it0, int n) {
  const iris_params& p = E->p;
  int it = it0;
  while (it < it0 + n) {
    if (graph_ready(E, it, it0 + n - it)) {
      int rc = graph_block(E, it, [&] {
        for (int j = 0; j < E->K; ++j) {
          launch_e<T>(E);
          launch_h<T>(E);
          launch_tfsf<T>(E, j, E->d_it);
          dft_sample<T>(E, j + 1 - p.to_fourier, E->d_it);
        }
      });
      if (rc) return rc;
      it += E->K;
      continue;
    }
    launch_e<T>(E);
    launch_h<T>(E);
    launch_tfsf<T>(E, it);
    if (it >= p.to_fourier && it % p.sample_fourier == 0) dft_sample<T>(E, it + 1 - p.to_fourier);
    ++it;
  }
  CK(cudaGetLastError());
  return IRIS_OK;
}

// Whether no DFT sample point lies on a plane the TF/SF corrections write
// (E at iz_min, H at iz_min-1 in variant 1 and at iz_min in variant 2): then
// k_tiny samples in the TF/SF phase.
static bool tiny_sample_merges(const iris_engine* E) {
  const int zm = E->src.iz_min;
  const int zh = E->src.variant == 1 ? zm - 1 : zm;
  for (const Seg& sg : E->segs) {
    long lo = sg.src, hi = sg.src;
    for (int cu = 0; cu < 2; ++cu)
      for (int cv = 0; cv < 2; ++cv) {
        const long q = sg.src + (cu ? (long)(sg.nu - 1) * sg.su : 0) + (cv ? (long)(sg.nv - 1) * sg.sv : 0);
        lo = std::min(lo, q);
        hi = std::max(hi, q);
      }
    const long z0 = lo / E->g.plane, z1 = hi / E->g.plane;
    const int zc = sg.field < 3 ? zm : zh;
    if (zc >= z0 && zc <= z1) return false;
  }
  return true;
}

// Steps it0 .. it0+n-1 with the persistent kernel: spans that end where the
// DFT ring fills (its commit runs between launches), after 1024 steps or at
// the TF/SF table's capacity; before each span k_tfsf_table evaluates its
// TF/SF corrections.
template <typename T> int step_persist(iris_engine* E, int it0, int n) {
  const iris_params& p = E->p;
  const int cap = E->src.variant != 0 ? E->tfv_cap : 1024;
  const bool merged = tiny_sample_merges(E);
  if (E->P > 0 && !E->d_sidx) {
    // flat table of the sample points: storage index * 8 + field
    std::vector<long> code((size_t)E->P);
    for (const Seg& sg : E->segs)
      for (long L = 0; L < (long)sg.nu * sg.nv; ++L) {
        const long v = L / sg.nu, u = L - v * sg.nu;
        code[(size_t)(sg.p0 + L)] = (sg.src + u * sg.su + v * sg.sv) * 8 + sg.field;
      }
    CK(cudaMalloc(&E->d_sidx, sizeof(long) * (size_t)E->P));
    CK(cudaMemcpy(E->d_sidx, code.data(), sizeof(long) * (size_t)E->P, cudaMemcpyHostToDevice));
  }
  int it = it0;
  while (it < it0 + n) {
    int span = 0, samples = 0;
    while (it + span < it0 + n && span < cap) {
      const int t = it + span;
      ++span;
      if (E->P > 0 && t >= p.to_fourier && t % p.sample_fourier == 0 && ++samples + E->nslot == E->K) break;
    }
    TinyArgs<T> A{};
    A.a = field_args<T>(E);
    A.s = E->src;
    A.tfv = E->d_tfv;
    A.merged = merged ? 1 : 0;
    A.sidx = E->d_sidx;
    A.segs = E->d_segs;
    A.nsegs = (int)E->segs.size();
    A.S = (typename V2<T>::t*)E->S;
    A.P = E->P;
    A.tk = E->d_tk;
    A.slot0 = E->nslot;
    A.it0 = it;
    A.n = span;
    A.to_fourier = p.to_fourier;
    A.sample_fourier = p.sample_fourier;
    A.dft = E->P > 0 ? 1 : 0;
    A.bar = (GridBar*)E->d_bar;
    A.err = E->d_err;
    void* args[] = {&A};
    {
      KTimer tm(E, IRIS_KC_PERSIST);
      if (E->src.variant != 0) {
        const long nt = (long)span * (p.nx + 2);
        k_tfsf_table<<<(unsigned)((nt + 127) / 128), 128, 0, E->st>>>(E->src, it, span, p.nx + 2, E->d_tfv);
      }
      CK(cudaMemsetAsync(E->d_bar, 0, sizeof(GridBar), E->st));
      const void* k = E->eps_complex ? (const void*)k_tiny<T, true> : (const void*)k_tiny<T, false>;
      CK(cudaLaunchCooperativeKernel(k, dim3(E->persist_blocks), dim3(E->persist_threads), args, 0, E->st));
    }
    E->nslot += samples;
    if (E->nslot == E->K) dft_flush(E);
    it += span;
  }
  CK(cudaGetLastError());
  return IRIS_OK;
}

int upload_material(iris_engine* E, const double* re, const double* im) {
  const iris_params& p = E->p;
  graph_reset(E);  // captured launches hold the old material pointer
  const Geo& g = E->g;
  const int nzs = p.hf - p.hi + 1;  // planes stored: hi..hf
  const long nxy = (long)(p.nx + 2) * (p.ny + 2);
  // 1/eps_bbox as a complex division (Smith's algorithm), for the default
  double c = p.eps_bbox_re, d = p.eps_bbox_im, ir, ii;
  if (std::fabs(c) >= std::fabs(d)) {
    const double r = d / c, den = c + d * r;
    ir = (1.0 + 0.0 * r) / den;
    ii = (0.0 - 1.0 * r) / den;
  } else {
    const double r = c / d, den = c * r + d;
    ir = (1.0 * r + 0.0) / den;
    ii = (0.0 * r - 1.0) / den;
  }
  bool cplx = false;
  if (re) {
    if (im)
      for (long i = nxy; i < nxy * (nzs + 1); ++i)
        if (im[i] != 0.0) { cplx = true; break; }
  } else {
    cplx = ii != 0.0;
  }
  if (E->eps) { cudaFree(E->eps); E->eps = nullptr; }
  if (nzs <= 0) { E->eps_complex = false; return IRIS_OK; }
  const long n = (long)nzs * g.plane;
  const size_t rsz = E->prec == IRIS_FP64 ? 8 : 4;
  const size_t bytes = (size_t)n * rsz * (cplx ? 2 : 1);
  CK(cudaMalloc(&E->eps, bytes));
  CK(cudaMemsetAsync(E->eps, 0, bytes, E->st));
  double* dre = nullptr;
  double* dim = nullptr;
  const size_t vb = sizeof(double) * (size_t)nxy * nzs;
  if (re) {
    // planes hi..hf of the host array (its plane 0 is hi-1)
    CK(cudaMalloc(&dre, vb));
    CK(cudaMemcpyAsync(dre, re + nxy, vb, cudaMemcpyHostToDevice, E->st));
    if (cplx) {
      CK(cudaMalloc(&dim, vb));
      CK(cudaMemcpyAsync(dim, im + nxy, vb, cudaMemcpyHostToDevice, E->st));
    }
  }
  const unsigned nb = (unsigned)((nxy * nzs + 255) / 256);
  if (E->prec == IRIS_FP64)
    k_material<double><<<nb, 256, 0, E->st>>>(dre, dim, g, nzs, ir, ii, p.aix, p.afx,
                                               cplx ? nullptr : (double*)E->eps, cplx ? (double2*)E->eps : nullptr);
  else
    k_material<float><<<nb, 256, 0, E->st>>>(dre, dim, g, nzs, ir, ii, p.aix, p.afx,
                                              cplx ? nullptr : (float*)E->eps, cplx ? (float2*)E->eps : nullptr);
  const cudaError_t e1 = cudaGetLastError();
  const cudaError_t e2 = cudaStreamSynchronize(E->st);
  if (dre) cudaFree(dre);
  if (dim) cudaFree(dim);
  if (e1 != cudaSuccess || e2 != cudaSuccess) return fail(IRIS_ECUDA, "material upload failed");
  E->eps_complex = cplx;
  return IRIS_OK;
}

// Builds the structure material on the device (k_material_gen); a real
// material, so eps_bbox must be real.
int generate_material(iris_engine* E, GenArgs G, const double* host_spheres) {
  const iris_params& p = E->p;
  if (p.eps_bbox_im != 0.0) return fail(IRIS_EINVAL, "material generators need a real eps_bbox");
  const int nzs = p.hf - p.hi + 1;
  if (nzs <= 0) return fail(IRIS_EINVAL, "no structure planes (hf < hi)");
  graph_reset(E);  // captured launches hold the old material pointer
  G.hi = p.hi;
  G.hf = p.hf;
  G.base = 1.0 / p.eps_bbox_re;
  if (E->eps) {
    CK(cudaStreamSynchronize(E->st));
    cudaFree(E->eps);
    E->eps = nullptr;
  }
  const Geo& g = E->g;
  const size_t rsz = E->prec == IRIS_FP64 ? 8 : 4;
  CK(cudaMalloc(&E->eps, (size_t)nzs * g.plane * rsz));
  CK(cudaMemsetAsync(E->eps, 0, (size_t)nzs * g.plane * rsz, E->st));
  SphereBox* dsph = nullptr;
  int *doff = nullptr, *dlst = nullptr;
  std::vector<SphereBox> boxes;
  if (G.kind == 1 && G.nsph > 0) {
    boxes.resize(G.nsph);
    for (int k = 0; k < G.nsph; ++k) {
      const double* q = host_spheres + 5 * k;
      const double cx = q[0], cy = q[1], cz = q[2], r = q[3];
      SphereBox& b = boxes[k];
      b.cx = cx;
      b.cy = cy;
      b.cz = cz;
      b.r2 = r * r;
      b.inv = 1.0 / q[4];
      b.zlo = std::max(p.hi, (int)std::floor(cz - r));
      b.zhi = std::min(p.hf, (int)std::ceil(cz + r));
      b.xlo = (int)std::floor(cx - r);
      b.lx = std::min(p.nx, (int)std::ceil(cx + r) - b.xlo + 1);
      b.ylo = (int)std::floor(cy - r);
      b.ly = std::min(p.ny, (int)std::ceil(cy + r) - b.ylo + 1);
    }
    CK(cudaMalloc(&dsph, sizeof(SphereBox) * G.nsph));
    CK(cudaMemcpyAsync(dsph, boxes.data(), sizeof(SphereBox) * G.nsph, cudaMemcpyHostToDevice, E->st));
    // bin the spheres per (plane, tile): the x (y) tiles a box touches are
    // those of the cells (x - xlo) mod nx < lx, wrapped into 1..nx
    const int ntx = (p.nx + GEN_TILE - 1) / GEN_TILE, nty = (p.ny + GEN_TILE - 1) / GEN_TILE;
    const long nbin = (long)nzs * ntx * nty;
    std::vector<std::vector<int>> tx(G.nsph), ty(G.nsph);
    long total = 0;
    for (int k = 0; k < G.nsph; ++k) {
      const SphereBox& b = boxes[k];
      auto tiles = [](int lo, int len, int n, std::vector<int>& out) {
        std::vector<char> hit((n + GEN_TILE - 1) / GEN_TILE, 0);
        for (int i = 0; i < len; ++i) hit[(((lo + i - 1) % n + n) % n) / GEN_TILE] = 1;
        for (int t = 0; t < (int)hit.size(); ++t)
          if (hit[t]) out.push_back(t);
      };
      tiles(b.xlo, b.lx, p.nx, tx[k]);
      tiles(b.ylo, b.ly, p.ny, ty[k]);
      if (b.zhi >= b.zlo) total += (long)(b.zhi - b.zlo + 1) * tx[k].size() * ty[k].size();
    }
    if (total < (1L << 26)) {
      std::vector<int> off(nbin + 1, 0), lst(std::max(1L, total));
      for (int k = 0; k < G.nsph; ++k)
        for (int z = boxes[k].zlo; z <= boxes[k].zhi; ++z)
          for (int ya : ty[k])
            for (int xa : tx[k]) ++off[((long)(z - p.hi) * nty + ya) * ntx + xa + 1];
      for (long b = 0; b < nbin; ++b) off[b + 1] += off[b];
      std::vector<int> fill(off.begin(), off.end() - 1);
      for (int k = 0; k < G.nsph; ++k)  // ascending within every bin
        for (int z = boxes[k].zlo; z <= boxes[k].zhi; ++z)
          for (int ya : ty[k])
            for (int xa : tx[k]) lst[fill[((long)(z - p.hi) * nty + ya) * ntx + xa]++] = k;
      CK(cudaMalloc(&doff, sizeof(int) * off.size()));
      CK(cudaMalloc(&dlst, sizeof(int) * lst.size()));
      CK(cudaMemcpyAsync(doff, off.data(), sizeof(int) * off.size(), cudaMemcpyHostToDevice, E->st));
      CK(cudaMemcpyAsync(dlst, lst.data(), sizeof(int) * lst.size(), cudaMemcpyHostToDevice, E->st));
      // the host vectors must outlive the copies
      CK(cudaStreamSynchronize(E->st));
      G.off = doff;
      G.lst = dlst;
      G.ntx = ntx;
      G.nty = nty;
    }
  }
  G.sph = dsph;
  const long n = (long)(p.nx + 2) * (p.ny + 2) * nzs;
  const unsigned nb = (unsigned)((n + 255) / 256);
  if (E->prec == IRIS_FP64) k_material_gen<double><<<nb, 256, 0, E->st>>>(G, g, (double*)E->eps);
  else k_material_gen<float><<<nb, 256, 0, E->st>>>(G, g, (float*)E->eps);
  const cudaError_t e1 = cudaGetLastError();
  const cudaError_t e2 = cudaStreamSynchronize(E->st);
  if (dsph) cudaFree(dsph);
  if (doff) cudaFree(doff);
  if (dlst) cudaFree(dlst);
  if (e1 != cudaSuccess || e2 != cudaSuccess) return fail(IRIS_ECUDA, "material generation failed");
  E->eps_complex = false;
  return IRIS_OK;
}

int build_dft(iris_engine* E) {
  const iris_params& p = E->p;
  bool single = true;
  for (int i = 0; i < 6; ++i)
    if (p.box1[i] != p.box2[i]) single = false;
  E->nboxes = single ? 1 : 2;
  bool on[3];
  if (p.nx != 1 && p.ny != 1) on[0] = on[1] = on[2] = true;
  else {
    on[0] = (p.ny == 1 && p.nx != 1);
    on[1] = (p.nx == 1 && p.ny != 1);
    on[2] = true;
  }
  if (E->dft_z_only) on[0] = on[1] = false;
  static const int comps[3][4] = {{1, 5, 2, 4}, {2, 3, 0, 5}, {0, 4, 1, 3}};  // (a,b,c,d) 0-based
  std::vector<FluxFace> faces(12);
  long P = 0;
  E->segs.clear();
  E->max_seg = 0;
  for (int b = 0; b < E->nboxes; ++b) {
    const int* bx = b == 0 ? p.box1 : p.box2;
    const int bxi = bx[0], bxf = bx[1], byi = bx[2], byf = bx[3], bzi = bx[4], bzf = bx[5];
    const int nbx = bxf + 1 - bxi, nby = byf + 1 - byi, nbz = bzf + 1 - bzi;
    for (int j = 0; j < 3; ++j) {
      FaceMap& F = E->fm[b][j];
      F = FaceMap();
      if (!on[j]) continue;
      F.active = true;
      for (int side = 0; side < 2; ++side) {
        long src, su, sv;
        int nu, nv;
        if (j == 0) {
          src = E->g.at(side ? bxf : bxi, byi, bzi); su = E->g.pitch; sv = E->g.plane; nu = nby; nv = nbz;
        } else if (j == 1) {
          src = E->g.at(bxi, side ? byf : byi, bzi); su = 1; sv = E->g.plane; nu = nbx; nv = nbz;
        } else {
          src = E->g.at(bxi, byi, side ? bzf : bzi); su = 1; sv = E->g.pitch; nu = nbx; nv = nby;
        }
        F.nu = nu;
        F.nv = nv;
        F.nloc = (long)nu * nv;
        for (int ip = 0; ip < 6; ++ip) {
          Seg s{};
          s.src = src; s.su = su; s.sv = sv; s.nu = nu; s.nv = nv; s.field = ip; s.p0 = P;
          E->segs.push_back(s);
          F.base[side][ip] = P;
          P += F.nloc;
          E->max_seg = std::max(E->max_seg, F.nloc);
        }
        FluxFace& ff = faces[6 * b + 2 * j + side];
        ff.pa = F.base[side][comps[j][0]];
        ff.pb = F.base[side][comps[j][1]];
        ff.pc = F.base[side][comps[j][2]];
        ff.pd = F.base[side][comps[j][3]];
        ff.n = F.nloc;
        ff.sign = side == 0 ? -1 : +1;
        ff.active = 1;
      }
    }
  }
  if (E->max_seg >= (1L << 31) - GATHER_BLOCK) return fail(IRIS_EINVAL, "a DFT face has 2^31 or more locations");
  E->P = P;
  E->host_faces = faces;
  if (E->member) return IRIS_OK;  // a batch member: the batch owns the DFT buffers
  return alloc_dft(E, faces.data(), 12);
}

}  // namespace

namespace iris {

void dft_flush(iris_engine* E) {
  if (E->nslot == 0) return;
  KTimer tm(E, IRIS_KC_DFT);
  const int nk = E->nslot;
  // the CUDA-core blocks read what they add to (on a failure the samples stay buffered)
  if (!E->dft_tc && fd_materialise(E)) return;
  if (E->prec == IRIS_FP64) {
    const int nwc = (E->p.nof + DFT64_WC - 1) / DFT64_WC;
    const long nblk = (E->P + 127) / 128;
    k_twiddle64<<<(nk * E->p.nof + 255) / 256, 256, 0, E->st>>>(E->d_tk, nk, E->d_fw, E->p.nof, E->d_wt64);
    k_dft_fp64<<<(unsigned)(nblk * nwc), 128, (size_t)nk * DFT64_WC * sizeof(double2), E->st>>>(
        (const double2*)E->S, E->P, nk, E->d_wt64, E->p.nof, nwc, E->p.dt, (double2*)E->fd);
  } else if (E->dft_tc) {
    const int ng = (E->p.nof + TC_NW - 1) / TC_NW, nch = (2 * nk + TC_KC - 1) / TC_KC;
    const long nt = (long)ng * nch * TC_BROWS * TC_KC;
    k_twiddle_tc<<<(unsigned)((nt + 255) / 256), 256, 0, E->st>>>(E->d_tk, 0, 0, nk, E->d_fw, E->p.nof, E->p.dt, ng,
                                                                   nch, E->d_wtc);
    WsArgs A{};
    A.S = (const float2*)E->S;
    A.P = E->P;
    A.nk = nk;
    A.Bt = E->d_wtc;
    A.fd = (float4*)E->fd;
    A.fd_zero = E->fd_zero;
    A.nof = E->p.nof;
    A.ngroups = ng;
    A.nitems = (E->P + TC_M - 1) / TC_M * ng;
    A.err = E->d_err;
    k_dft_ws_commit<<<(unsigned)std::min<long>(A.nitems, E->ws_blocks), WsCfg<false>::THREADS, WS_SMEM, E->st>>>(A);
    E->fd_zero = false;  // every accumulator of every frequency has been written
  } else {
    const int nt = nk * E->p.nof;
    k_twiddle<<<(nt + 255) / 256, 256, 0, E->st>>>(E->d_tk, 0, 0, nk, E->d_fw, E->p.nof, E->p.dt, E->d_wt);
    const int nwc = (E->p.nof + DFT_TW - 1) / DFT_TW;
    const long nblk = (E->P + DFT_TP - 1) / DFT_TP;
    k_dft_fp32<float4><<<(unsigned)(nblk * nwc), DFT_THREADS, 0, E->st>>>((const float2*)E->S, E->P, nk, E->d_wt, E->p.nof, nwc,
                                                        (float4*)E->fd);
  }
  E->nslot = 0;
}

int fd_materialise(iris_engine* E) {
  if (!E->fd_zero) return IRIS_OK;
  CK(cudaMemsetAsync(E->fd, 0, (size_t)E->P * E->p.nof * 16, E->st));
  E->fd_zero = false;
  return IRIS_OK;
}

// A whole DFT block of steps from it on can be replayed from a graph: every
// step of it is sampled and the block starts with an empty ring.
bool graph_ready(const iris_engine* E, int it, int left) {
  const iris_params& p = E->p;
  // the fused passes swap buffers every step: an even block brings them back
  return p.graph && !E->timing && (!E->fused || E->K % 2 == 0) && E->P > 0 && E->nslot == 0 &&
         p.sample_fourier == 1 && it >= p.to_fourier && left >= E->K;
}

void graph_reset(iris_engine* E) {
  if (E->gexec) cudaGraphExecDestroy(E->gexec);
  E->gexec = nullptr;
}

// Steps it .. it+K-1 from the engine's graph of one DFT block (captured on
// first use from record(), which issues the K steps with step offsets
// 0 .. K-1 relative to the device-resident base d_it, the block's sample
// flush, and the base's advance by K).
int graph_block(iris_engine* E, int it, const std::function<void()>& record) {
  if (!E->d_it) {
    CK(cudaMalloc(&E->d_it, sizeof(int)));
    E->dev_it = -1;
  }
  if (E->dev_it != it) k_set_int<<<1, 1, 0, E->st>>>(E->d_it, it);
  if (!E->gexec) {
    // the captured commit is replayed for every block: it must read the sums
    if (int rc = fd_materialise(E)) return rc;
    cudaGraph_t gr = nullptr;
    CK(cudaStreamBeginCapture(E->st, cudaStreamCaptureModeRelaxed));
    record();
    k_add_int<<<1, 1, 0, E->st>>>(E->d_it, E->K);
    const cudaError_t ec = cudaStreamEndCapture(E->st, &gr);
    if (ec != cudaSuccess) return fail(IRIS_ECUDA, std::string("graph capture: ") + cudaGetErrorString(ec));
    const cudaError_t ei = cudaGraphInstantiate(&E->gexec, gr, 0);
    cudaGraphDestroy(gr);
    if (ei != cudaSuccess) {
      E->gexec = nullptr;
      return fail(IRIS_ECUDA, std::string("graph instantiation: ") + cudaGetErrorString(ei));
    }
  }
  CK(cudaGraphLaunch(E->gexec, E->st));
  E->dev_it = it + E->K;
  return IRIS_OK;
}

// DFT buffers for E->P sample points: accumulators, the K-slot sample ring,
// twiddles, the flux faces (nfaces FluxFace) and the flux output.
int alloc_dft(iris_engine* E, const FluxFace* faces, int nfaces) {
  const iris_params& p = E->p;
  const long P = E->P;
  // block length K: samples buffered before one accumulation pass
  size_t freeb = 0, totb = 0;
  CK(cudaMemGetInfo(&freeb, &totb));
  const size_t fd_bytes = (size_t)P * p.nof * sizeof(double2);
  if (fd_bytes > freeb) return fail(IRIS_ENOMEM, "DFT accumulators exceed free device memory");
  // FP64: at most 256 slots (its block kernel stages K x 8 twiddles in 32 KB
  // of shared memory), 32 by default.  FP32: up to 512, the default: a block
  // reads and writes the FP64 accumulators once, so a longer block moves
  // fewer accumulator bytes per sample.  The ring takes at most half of the
  // memory left after the accumulators.
  const int kmax = E->prec == IRIS_FP64 ? 256 : 512;
  int K = std::min(kmax, p.dft_block > 0 ? p.dft_block : (E->prec == IRIS_FP64 ? 32 : 512));
  const size_t slot_bytes = std::max<size_t>(1, (size_t)P * E->esz);
  const size_t budget = (freeb - fd_bytes) / 2;
  while (K > 1 && (size_t)K * slot_bytes > budget) K /= 2;
  E->K = std::max(1, K);
  E->nslot = 0;
  CK(cudaMalloc(&E->fd, std::max<size_t>(fd_bytes, 16)));
  E->fd_zero = true;  // zeroed when first read as it lies, never for the tensor-core path
  CK(cudaMalloc(&E->S, (size_t)E->K * slot_bytes));
  CK(cudaMalloc(&E->d_tk, sizeof(int) * E->K));
  CK(cudaMalloc(&E->d_fw, sizeof(double) * p.nof));
  CK(cudaMemcpy(E->d_fw, E->fw.data(), sizeof(double) * p.nof, cudaMemcpyHostToDevice));
  if (E->prec == IRIS_FP32) CK(cudaMalloc(&E->d_wt, sizeof(float2) * (size_t)E->K * p.nof));
  if (E->prec == IRIS_FP64) CK(cudaMalloc(&E->d_wt64, sizeof(double2) * (size_t)E->K * p.nof));
  E->dft_tc = E->prec == IRIS_FP32 && p.dft_kernel != IRIS_DFT_KERNEL_CUDA;
  E->flux_faces.assign(faces, faces + nfaces);
  if (E->dft_tc) {
    const int ng = (p.nof + TC_NW - 1) / TC_NW, nch = (2 * E->K + TC_KC - 1) / TC_KC;
    CK(cudaMalloc(&E->d_wtc, sizeof(float) * (size_t)ng * nch * 2 * TC_BROWS * TC_KC));
    CK(cudaFuncSetAttribute(k_dft_ws_commit, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)WS_SMEM));
    CK(cudaFuncSetAttribute(k_dft_ws_flux, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)WS_SMEM));
    int nsm = 0;
    CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, E->device));
    E->ws_blocks = std::max(1, nsm);  // one persistent CTA per SM (its TMEM takes all 512 columns)
    long maxt = 1;
    for (int s = 0; s + 6 <= nfaces; s += 6) maxt = std::max(maxt, (long)flux_tiles(faces + s).start[6]);
    CK(cudaMalloc(&E->d_part, sizeof(double) * 4 * (size_t)maxt * p.nof));
  }
  if (!E->segs.empty()) {
    CK(cudaMalloc(&E->d_segs, sizeof(Seg) * E->segs.size()));
    CK(cudaMemcpy(E->d_segs, E->segs.data(), sizeof(Seg) * E->segs.size(), cudaMemcpyHostToDevice));
  }
  CK(cudaMalloc(&E->d_faces, sizeof(FluxFace) * nfaces));
  CK(cudaMemcpy(E->d_faces, faces, sizeof(FluxFace) * nfaces, cudaMemcpyHostToDevice));
  CK(cudaMalloc(&E->d_J, sizeof(double) * 6 * p.nof));
  CK(cudaMallocHost(&E->h_J, sizeof(double) * 6 * p.nof));
  return IRIS_OK;
}

void free_engine(iris_engine* E) {
  void* ptrs[] = {E->e, E->h, E->pml_d[0], E->pml_d[1], E->pml_b[0], E->pml_b[1], E->coef, E->eps, E->d_segs,
                  E->S, E->d_tk, E->d_fw, E->fd, E->d_wt, E->d_faces, E->d_J, E->e2, E->h2, E->pml_d2[0],
                  E->pml_d2[1], E->d_err, E->d_it, E->d_wtc, E->d_wt64, E->d_part, E->d_bar, E->d_stage,
                  E->d_tfv, E->d_sidx};
  for (void* q : ptrs)
    if (q) cudaFree(q);
  if (E->h_J) cudaFreeHost(E->h_J);
  graph_reset(E);
  for (int k = 0; k < IRIS_NKC; ++k)
    for (auto& pr : E->ev[k]) {
      cudaEventDestroy(pr.first);
      cudaEventDestroy(pr.second);
    }
  if (E->t0) cudaEventDestroy(E->t0);
  if (E->t1) cudaEventDestroy(E->t1);
  if (E->fz_fork) cudaEventDestroy(E->fz_fork);
  if (E->fz_join) cudaEventDestroy(E->fz_join);
  if (E->st2) cudaStreamDestroy(E->st2);
  if (E->st) cudaStreamDestroy(E->st);
}


void one_step(iris_engine* E, int it, bool dft) {
  const iris_params& p = E->p;
  const bool sampled = dft && it >= p.to_fourier && it % p.sample_fourier == 0;
  if (E->fused) {
    fused_one(E, it, nullptr, sampled);
  } else if (E->prec == IRIS_FP64) {
    launch_e<double>(E);
    launch_h<double>(E);
    launch_tfsf<double>(E, it);
    if (sampled) dft_sample<double>(E, it + 1 - p.to_fourier);
  } else {
    launch_e<float>(E);
    launch_h<float>(E);
    launch_tfsf<float>(E, it);
    if (sampled) dft_sample<float>(E, it + 1 - p.to_fourier);
  }
}

// packed: rows of nx+2 cells back to back (no 128-byte alignment of x = 1),
// for cells whose rows are short; component arrays stay 128-byte aligned.
int create_engine(const iris_params* pin, const double* fw, bool member, bool z_only, iris_engine** out,
                  bool packed) {
  clear_error();
  if (!pin || !fw || !out) return fail(IRIS_EINVAL, "null argument");
  *out = nullptr;
  int rc = validate(*pin);
  if (rc) return rc;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(IRIS_ENODEV, "no CUDA device");
  if (pin->device < 0 || pin->device >= ndev) return fail(IRIS_EINVAL, "device ordinal out of range");
  iris_engine* E = new iris_engine();
  E->p = *pin;
  E->member = member;
  E->dft_z_only = z_only || pin->dft_faces == IRIS_DFT_Z;
  const iris_params& p = E->p;
  E->fw.assign(fw, fw + p.nof);
  E->prec = p.precision;
  E->esz = p.precision == IRIS_FP64 ? 16 : 8;
  E->device = p.device;
  auto bail = [&](int code) {
    free_engine(E);
    delete E;
    return code;
  };
  if (cudaSetDevice(E->device) != cudaSuccess) return bail(fail(IRIS_ECUDA, "cudaSetDevice failed"));
  if (cudaStreamCreateWithFlags(&E->st, cudaStreamNonBlocking) != cudaSuccess)
    return bail(fail(IRIS_ECUDA, "cudaStreamCreate failed"));
  // geometry: x = 1 on a 128-byte boundary, or packed rows
  Geo& g = E->g;
  g.nx = p.nx;
  g.ny = p.ny;
  g.nz = p.nz;
  const int align = (int)(128 / E->esz);
  g.xo = packed ? 0 : align - 1;
  g.pitch = packed ? (long)p.nx + 2 : ((long)(g.xo + p.nx + 2) + align - 1) / align * align;
  g.plane = g.pitch * (p.ny + 2);
  g.comp = (g.plane * (p.nz + 2) + align - 1) / align * align;
  const size_t fbytes = (size_t)3 * g.comp * E->esz;
  if (cudaMalloc(&E->e, fbytes) != cudaSuccess || cudaMalloc(&E->h, fbytes) != cudaSuccess)
    return bail(fail(IRIS_ENOMEM, "field allocation failed"));
  cudaMemsetAsync(E->e, 0, fbytes, E->st);
  cudaMemsetAsync(E->h, 0, fbytes, E->st);
  E->nbot = p.pmlzi;
  E->ntop = p.nz - p.pmlzf + 1;
  for (int s = 0; s < 2; ++s) {
    E->pcomp[s] = (long)p.nx * p.ny * (s == 0 ? E->nbot : E->ntop);
    const size_t b = (size_t)3 * E->pcomp[s] * E->esz;
    if (cudaMalloc(&E->pml_d[s], b) != cudaSuccess || cudaMalloc(&E->pml_b[s], b) != cudaSuccess)
      return bail(fail(IRIS_ENOMEM, "UPML allocation failed"));
    cudaMemsetAsync(E->pml_d[s], 0, b, E->st);
    cudaMemsetAsync(E->pml_b[s], 0, b, E->st);
  }
  make_coef(p, E->coef_h);
  {
    const size_t n = E->coef_h.size();
    if (E->prec == IRIS_FP64) {
      if (cudaMalloc(&E->coef, n * 8) != cudaSuccess) return bail(fail(IRIS_ENOMEM, "coef allocation failed"));
      cudaMemcpy(E->coef, E->coef_h.data(), n * 8, cudaMemcpyHostToDevice);
    } else {
      std::vector<float> f(n);
      for (size_t i = 0; i < n; ++i) f[i] = (float)E->coef_h[i];
      if (cudaMalloc(&E->coef, n * 4) != cudaSuccess) return bail(fail(IRIS_ENOMEM, "coef allocation failed"));
      cudaMemcpy(E->coef, f.data(), n * 4, cudaMemcpyHostToDevice);
    }
  }
  // Bloch phases cdexp(+-ci*ak) (code/boundary.f90:175,205,237,270,301,334)
  const double ak[3][2] = {{p.akx_re, p.akx_im}, {p.aky_re, p.aky_im}, {p.akz_re, p.akz_im}};
  for (int a = 0; a < 3; ++a)
    for (int sgn = 0; sgn < 2; ++sgn) {
      const double s = sgn == 0 ? 1.0 : -1.0;
      const double ar = -s * ak[a][1], ai = s * ak[a][0];  // (+-ci)*ak
      const double m = std::exp(ar);
      E->ph[3 * sgn + a][0] = m * std::cos(ai);
      E->ph[3 * sgn + a][1] = m * std::sin(ai);
    }
  // launch shapes
  const int bx = std::min(32, p2ceil(p.nx));
  const int by = std::min(256 / bx, p2ceil(p.ny));
  const int bz = std::min(std::min(256 / (bx * by), p2ceil(p.nz)), 64);  // blockDim.z <= 64
  E->blk = dim3(bx, by, bz);
  E->grd = dim3((p.nx + bx - 1) / bx, (p.ny + by - 1) / by, (p.nz + bz - 1) / bz);
  E->src = make_src(p);
  E->tf_blk = dim3(64);
  E->tf_grd = dim3((p.nx + 2 + 63) / 64, (p.ny + 2 + TFSF_YCH - 1) / TFSF_YCH);
  // Small grids step with the persistent kernel (asked for, or by default
  // when the device runs cooperative launches: FP64 grids of at most
  // IRIS_PERSISTENT_MAX_CELLS cells, FP32 grids of at most
  // IRIS_PERSISTENT_MAX_CELLS_FP32: up to those sizes it steps faster than
  // the split passes); otherwise FP32 steps with the fused E+H pass unless the split or
  // streamed passes are asked for, or unless the fused pass's 32 x 16 tiles
  // would leave more than half of their threads idle on the grid's x-y
  // plane (rows or columns short of a tile: the split passes then); FP64
  // steps with the split passes.
  {
    int coop = 0, nsm = 0, occ = 0;
    cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, E->device);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, E->device);
    const long cells = (long)p.nx * p.ny * p.nz;
    const long dflt = E->prec == IRIS_FP64 ? IRIS_PERSISTENT_MAX_CELLS : IRIS_PERSISTENT_MAX_CELLS_FP32;
    const bool want = !member && 3 * cells < (1L << 31) &&
                      (p.stencil == IRIS_STENCIL_PERSISTENT || (p.stencil == IRIS_STENCIL_DEFAULT && cells <= dflt));
    if (want && coop && nsm > 0) {
      // the widest CTA that still gives every SM at least one work item a
      // thread (three a cell in FP64); one CTA per SM at most (the FP64
      // pipes are per SM), no more than the work items need
      const long items = (E->prec == IRIS_FP64 ? 3 : 1) * cells;
      int thr = TINY_MIN_THREADS;
      while (thr < TINY_MAX_THREADS && items >= 2L * thr * nsm) thr *= 2;
      const void* k = E->prec == IRIS_FP64 ? (const void*)k_tiny<double, false> : (const void*)k_tiny<float, false>;
      const void* kc = E->prec == IRIS_FP64 ? (const void*)k_tiny<double, true> : (const void*)k_tiny<float, true>;
      int o1 = 0, o2 = 0;
      if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o1, k, thr, 0) == cudaSuccess &&
          cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o2, kc, thr, 0) == cudaSuccess)
        occ = std::min(o1, o2);
      const long need = (items + thr - 1) / thr;
      E->persist_threads = thr;
      E->persist_blocks = (int)std::max(1L, std::min<long>(need, (long)nsm * std::min(occ, 1)));
      E->persist = occ >= 1;
    }
    if (p.stencil == IRIS_STENCIL_PERSISTENT && !E->persist)
      return bail(fail(IRIS_EINVAL, "the persistent stencil needs cooperative launches on this device and "
                                    "fewer than 2^31 / 3 cells"));
    if (E->persist && cudaMalloc(&E->d_bar, 64) != cudaSuccess)
      return bail(fail(IRIS_ENOMEM, "barrier allocation failed"));
    if (E->persist && E->src.variant != 0) {
      // TF/SF table of a span: at most 1024 steps and 8 MB
      E->tfv_cap = (int)std::max(1L, std::min(1024L, (8L << 20) / (32L * (p.nx + 2))));
      if (cudaMalloc(&E->d_tfv, sizeof(TfsfVal) * (size_t)E->tfv_cap * (p.nx + 2)) != cudaSuccess)
        return bail(fail(IRIS_ENOMEM, "TF/SF table allocation failed"));
    }
  }
  E->fused = !E->persist && E->prec == IRIS_FP32 &&
             (p.stencil == IRIS_STENCIL_FUSED || (p.stencil == IRIS_STENCIL_DEFAULT && fused_fill(p.nx, p.ny) >= 0.5));
  if (E->fused) {
    if (cudaMalloc(&E->e2, fbytes) != cudaSuccess || cudaMalloc(&E->h2, fbytes) != cudaSuccess)
      return bail(fail(IRIS_ENOMEM, "second field buffers: allocation failed"));
    cudaMemsetAsync(E->e2, 0, fbytes, E->st);
    cudaMemsetAsync(E->h2, 0, fbytes, E->st);
    for (int s = 0; s < 2; ++s) {
      const size_t b = (size_t)3 * E->pcomp[s] * E->esz;
      if (cudaMalloc(&E->pml_d2[s], b) != cudaSuccess) return bail(fail(IRIS_ENOMEM, "UPML allocation failed"));
      cudaMemsetAsync(E->pml_d2[s], 0, b, E->st);
    }
    // z chunks: planes pmlzi+1 .. pmlzf-2 (the last chunk's extra plane,
    // whose E' its H' needs, is then still outside the slabs) by the kernel
    // without slab code, the slabs with the plane next to each by the other
    const long tiles = (long)((p.nx + FZ_OX - 1) / FZ_OX) * ((p.ny + FZ_OY - 1) / FZ_OY);
    const int ia = p.pmlzi + 1, ib = p.pmlzf - 2;
    for (int part = 0; part < 2; ++part) E->fzr[part].clear();
    if (ib >= ia) {
      fused_chunks(E->fzr[0], ia, ib, tiles);
      fused_chunks(E->fzr[1], 1, ia - 1, tiles);
      fused_chunks(E->fzr[1], ib + 1, p.nz, tiles);
    } else {
      fused_chunks(E->fzr[1], 1, p.nz, tiles);
    }
    E->fblk = dim3(FZ_X, FZ_Y, 1);
    if (cudaStreamCreateWithFlags(&E->st2, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&E->fz_fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&E->fz_join, cudaEventDisableTiming) != cudaSuccess)
      return bail(fail(IRIS_ECUDA, "fused pass: stream creation failed"));
    for (const void* kf : {(const void*)k_fused<false, true, long>, (const void*)k_fused<true, true, long>,
                           (const void*)k_fused<false, true, int>, (const void*)k_fused<true, true, int>})
      if (cudaFuncSetAttribute(kf, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)FZ_UPML_SMEM) != cudaSuccess)
        return bail(fail(IRIS_ECUDA, "fused pass: shared memory configuration failed"));
    E->fgrd = dim3((p.nx + FZ_OX - 1) / FZ_OX, (p.ny + FZ_OY - 1) / FZ_OY, 1);
    E->fz_i32 = 3 * E->g.comp < (1L << 31);
  }
  if (cudaMalloc(&E->d_err, sizeof(int)) != cudaSuccess) return bail(fail(IRIS_ENOMEM, "allocation failed"));
  cudaMemsetAsync(E->d_err, 0, sizeof(int), E->st);
  E->stream = E->prec == IRIS_FP32 && p.stencil == IRIS_STENCIL_STREAM && !packed;
  if (E->stream) {
    if (cudaFuncSetAttribute(k_stream_e, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)STREAM_SMEM_E) !=
            cudaSuccess ||
        cudaFuncSetAttribute(k_stream_h, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)STREAM_SMEM_H) !=
            cudaSuccess)
      return bail(fail(IRIS_ECUDA, "streamed stencil: shared memory opt-in failed"));
    E->sgrd = dim3((p.nx + SX - 1) / SX, (p.ny + SY - 1) / SY, (p.nz + SZC - 1) / SZC);
  }
  rc = upload_material(E, nullptr, nullptr);  // the reference's default material
  if (rc) return bail(rc);
  rc = build_dft(E);
  if (rc) return bail(rc);
  if (cudaStreamSynchronize(E->st) != cudaSuccess) return bail(fail(IRIS_ECUDA, "initialisation failed"));
  *out = E;
  return IRIS_OK;
}

}  // namespace iris

long iris::engine_npts(const iris_engine* E, int box, int j) {
  if (box < 0 || box >= E->nboxes || j < 1 || j > 3) return 0;
  const FaceMap& F = E->fm[box][j - 1];
  return F.active ? 12 * F.nloc : 0;
}

// Status of the engine's bounded device waits: IRIS_ETIMEOUT once a kernel
// gave up on one (the stream is synchronised first).
// The word is cleared once reported.
static int stream_status(iris_engine* E) {
  if (!E->d_err) return IRIS_OK;
  int h = 0;
  CK(cudaMemcpyAsync(&h, E->d_err, sizeof(int), cudaMemcpyDeviceToHost, E->st));
  CK(cudaStreamSynchronize(E->st));
  if (!h) return IRIS_OK;
  CK(cudaMemsetAsync(E->d_err, 0, sizeof(int), E->st));
  CK(cudaStreamSynchronize(E->st));
  const char* what = h == 1   ? "a streamed E pass gave up waiting for its staged plane"
                     : h == 2 ? "a streamed H pass gave up waiting for its staged plane"
                     : h == 3 ? "the tensor-core DFT block gave up waiting"
                     : h == 5 ? "the tensor-core flux read gave up waiting"
                     : h == 6 ? "the persistent step kernel gave up at a grid barrier"
                              : "the wait check gave up (as it must)";
  return fail(IRIS_ETIMEOUT, what);
}

// The flux of one face set.  FP32 mode on the tensor cores: over the
// accumulators plus the samples still in the ring, which stay there
// (k_twiddle_tc for the pending samples, k_dft_ws_flux, k_flux_sum).  Otherwise
// the ring is committed first and k_flux reads the accumulators.
int iris::read_flux(iris_engine* E, int set, double* J) {
  const iris_params& p = E->p;
  const double scale = p.eps0 * p.Q / (2.0 * p.dt);
  const FluxFace* f6 = E->flux_faces.data() + 6 * set;
  const FluxTiles ft = flux_tiles(f6);
  const int ng = (p.nof + TC_NW - 1) / TC_NW;
  if (E->dft_tc) {
    KTimer tm(E, IRIS_KC_FLUX);
    const int nk = E->nslot;
    if (nk > 0) {
      const int nch = (2 * nk + TC_KC - 1) / TC_KC;
      const long nt = (long)ng * nch * TC_BROWS * TC_KC;
      k_twiddle_tc<<<(unsigned)((nt + 255) / 256), 256, 0, E->st>>>(E->d_tk, 0, 0, nk, E->d_fw, p.nof, p.dt, ng, nch,
                                                                     E->d_wtc);
    }
    if (ft.start[6] > 0) {
      WsArgs A{};
      A.S = (const float2*)E->S;
      A.P = E->P;
      A.nk = nk;
      A.Bt = E->d_wtc;
      A.fd = (float4*)E->fd;
      A.fd_zero = E->fd_zero;
      A.nof = p.nof;
      A.ngroups = ng;
      A.nitems = (long)ft.start[6] * ng;
      A.faces = E->d_faces + 6 * set;
      A.ft = ft;
      A.part = E->d_part;
      A.err = E->d_err;
      k_dft_ws_flux<<<(unsigned)std::min<long>(A.nitems, E->ws_blocks), WsCfg<true>::THREADS, WS_SMEM, E->st>>>(A);
    }
    k_flux_sum<<<dim3(p.nof, 6), 256, 0, E->st>>>(E->d_part, ft, E->d_faces + 6 * set, p.nof, scale, E->d_J);
  } else {
    dft_flush(E);
    if (int rc = fd_materialise(E)) return rc;  // no block committed yet
    KTimer tm(E, IRIS_KC_FLUX);
    if (E->prec == IRIS_FP64)
      k_flux<double2><<<dim3(p.nof, 6), 256, 0, E->st>>>((const double2*)E->fd, E->P, E->d_faces + 6 * set, p.nof,
                                                          scale, E->d_J);
    else
      k_flux<float4><<<dim3(p.nof, 6), 256, 0, E->st>>>((const float4*)E->fd, E->P, E->d_faces + 6 * set, p.nof, scale,
                                                         E->d_J);
  }
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(E->h_J, E->d_J, sizeof(double) * 6 * p.nof, cudaMemcpyDeviceToHost, E->st));
  CK(cudaStreamSynchronize(E->st));
  int rc = stream_status(E);
  if (rc) return rc;
  bool finite = true;
  for (int k = 0; k < 6 * p.nof; ++k) {
    J[k] = E->h_J[k];
    if (!std::isfinite(J[k])) finite = false;
  }
  return finite ? IRIS_OK : fail(IRIS_ENAN, "non-finite flux");
}

extern "C" {

int iris_create(const iris_params* pin, const double* fw, iris_engine** out) {
  iris::NvtxRange nvtx_("iris_create");
  return create_engine(pin, fw, false, false, out);
}

void iris_destroy(iris_engine* E) {
  if (!E) return;
  cudaSetDevice(E->device);
  cudaStreamSynchronize(E->st);
  free_engine(E);
  delete E;
}

int iris_set_material(iris_engine* E, const double* re, const double* im) {
  clear_error();
  if (!E || !re) return fail(IRIS_EINVAL, "null argument");
  CK(cudaSetDevice(E->device));
  CK(cudaStreamSynchronize(E->st));
  return upload_material(E, re, im);
}

int iris_material_spheres(iris_engine* E, int n, const double* spheres) {
  clear_error();
  if (!E || n < 0 || (n > 0 && !spheres)) return fail(IRIS_EINVAL, "bad argument");
  for (int k = 0; k < n; ++k)
    if (!(spheres[5 * k + 3] >= 0.0) || !(spheres[5 * k + 4] != 0.0) || !std::isfinite(spheres[5 * k]) ||
        !std::isfinite(spheres[5 * k + 1]) || !std::isfinite(spheres[5 * k + 2]) ||
        !std::isfinite(spheres[5 * k + 3]) || spheres[5 * k + 3] > 1e6)
      return fail(IRIS_EINVAL, "sphere " + std::to_string(k) + ": centre, radius (0..1e6) or eps invalid");
  CK(cudaSetDevice(E->device));
  GenArgs G{};
  G.kind = 1;
  G.nsph = n;
  return generate_material(E, G, spheres);
}

int iris_material_pattern(iris_engine* E, unsigned long long seed, double fill, double eps_in, double eps_out) {
  clear_error();
  if (!E || eps_in == 0.0 || eps_out == 0.0) return fail(IRIS_EINVAL, "bad argument");
  CK(cudaSetDevice(E->device));
  GenArgs G{};
  G.kind = 2;
  G.seed = seed;
  G.fill = fill;
  G.v_in = 1.0 / eps_in;
  G.v_out = 1.0 / eps_out;
  return generate_material(E, G, nullptr);
}

int iris_material_design(iris_engine* E, unsigned long long seed, const int region[4], double emin, double emax) {
  clear_error();
  if (!E || !region) return fail(IRIS_EINVAL, "bad argument");
  const iris_params& p = E->p;
  if (region[0] < 1 || region[1] > p.nx || region[0] > region[1] || region[2] < 1 || region[3] > p.ny ||
      region[2] > region[3])
    return fail(IRIS_EINVAL, "design region must lie in [1,nx] x [1,ny]");
  CK(cudaSetDevice(E->device));
  GenArgs G{};
  G.kind = 3;
  G.seed = seed;
  G.x0 = region[0];
  G.x1 = region[1];
  G.y0 = region[2];
  G.y1 = region[3];
  G.emin = emin;
  G.emax = emax;
  return generate_material(E, G, nullptr);
}

int iris_get_material(iris_engine* E, double* re, double* im) {
  clear_error();
  if (!E || !re || !im) return fail(IRIS_EINVAL, "bad argument");
  CK(cudaSetDevice(E->device));
  const iris_params& p = E->p;
  const int nzs = p.hf - p.hi + 1;
  if (nzs <= 0 || !E->eps) return IRIS_OK;
  const long n = (long)(p.nx + 2) * (p.ny + 2) * nzs;
  double* d = nullptr;
  CK(cudaMalloc(&d, sizeof(double) * 2 * n));
  const unsigned nb = (unsigned)((n + 255) / 256);
  if (E->prec == IRIS_FP64) k_material_get<double><<<nb, 256, 0, E->st>>>(E->eps, E->eps_complex, E->g, nzs, d, d + n);
  else k_material_get<float><<<nb, 256, 0, E->st>>>(E->eps, E->eps_complex, E->g, nzs, d, d + n);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(re, d, sizeof(double) * n, cudaMemcpyDeviceToHost, E->st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(im, d + n, sizeof(double) * n, cudaMemcpyDeviceToHost, E->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(E->st);
  cudaFree(d);
  if (e != cudaSuccess) return fail(IRIS_ECUDA, std::string("iris_get_material: ") + cudaGetErrorString(e));
  return IRIS_OK;
}

int iris_step(iris_engine* E, int it0, int nsteps) {
  iris::NvtxRange nvtx_("iris_step");
  clear_error();
  if (!E || nsteps < 0) return fail(IRIS_EINVAL, "bad argument");
  CK(cudaSetDevice(E->device));
  if (E->persist)
    return E->prec == IRIS_FP64 ? step_persist<double>(E, it0, nsteps) : step_persist<float>(E, it0, nsteps);
  if (E->fused) return step_fused(E, it0, nsteps);
  return E->prec == IRIS_FP64 ? step_t<double>(E, it0, nsteps) : step_t<float>(E, it0, nsteps);
}

int iris_sync(iris_engine* E) {
  if (!E) return fail(IRIS_EINVAL, "null engine");
  CK(cudaSetDevice(E->device));
  CK(cudaStreamSynchronize(E->st));
  CK(cudaGetLastError());
  return stream_status(E);
}

int iris_flux(iris_engine* E, int box, double* J) {
  iris::NvtxRange nvtx_("iris_flux");
  clear_error();
  if (!E || !J || box < 0 || box > 1) return fail(IRIS_EINVAL, "bad argument");
  CK(cudaSetDevice(E->device));
  if (box >= E->nboxes) box = 0;  // a single box: the second one is the same box
  return read_flux(E, box, J);
}

int iris_get_field(iris_engine* E, int which, double* re, double* im) {
  clear_error();
  if (!E || !re || !im || (which != IRIS_E && which != IRIS_H)) return fail(IRIS_EINVAL, "bad argument");
  CK(cudaSetDevice(E->device));
  const Geo& g = E->g;
  const size_t n = (size_t)3 * g.comp;
  std::vector<unsigned char> buf(n * E->esz);
  CK(cudaMemcpyAsync(buf.data(), which == IRIS_E ? E->e : E->h, n * E->esz, cudaMemcpyDeviceToHost, E->st));
  CK(cudaStreamSynchronize(E->st));
  for (int z = 0; z <= g.nz + 1; ++z)
    for (int y = 0; y <= g.ny + 1; ++y)
      for (int x = 0; x <= g.nx + 1; ++x)
        for (int c = 0; c < 3; ++c) {
          const long r = c + 3L * (x + (long)(g.nx + 2) * (y + (long)(g.ny + 2) * z));
          const long s = c * g.comp + g.at(x, y, z);
          if (E->prec == IRIS_FP64) {
            re[r] = ((const double*)buf.data())[2 * s];
            im[r] = ((const double*)buf.data())[2 * s + 1];
          } else {
            re[r] = ((const float*)buf.data())[2 * s];
            im[r] = ((const float*)buf.data())[2 * s + 1];
          }
        }
  return IRIS_OK;
}

int iris_set_field(iris_engine* E, int which, const double* re, const double* im) {
  clear_error();
  if (!E || !re || !im || (which != IRIS_E && which != IRIS_H)) return fail(IRIS_EINVAL, "bad argument");
  CK(cudaSetDevice(E->device));
  const Geo& g = E->g;
  const size_t n = (size_t)3 * g.comp;
  std::vector<unsigned char> buf(n * E->esz, 0);
  for (int z = 0; z <= g.nz + 1; ++z)
    for (int y = 0; y <= g.ny + 1; ++y)
      for (int x = 0; x <= g.nx + 1; ++x)
        for (int c = 0; c < 3; ++c) {
          const long r = c + 3L * (x + (long)(g.nx + 2) * (y + (long)(g.ny + 2) * z));
          const long s = c * g.comp + g.at(x, y, z);
          if (E->prec == IRIS_FP64) {
            ((double*)buf.data())[2 * s] = re[r];
            ((double*)buf.data())[2 * s + 1] = im[r];
          } else {
            ((float*)buf.data())[2 * s] = (float)re[r];
            ((float*)buf.data())[2 * s + 1] = (float)im[r];
          }
        }
  CK(cudaMemcpyAsync(which == IRIS_E ? E->e : E->h, buf.data(), n * E->esz, cudaMemcpyHostToDevice, E->st));
  CK(cudaStreamSynchronize(E->st));
  return IRIS_OK;
}

static int pml_io(iris_engine* E, int which, int slab, double* re, double* im, const double* cre, const double* cim) {
  if (!E || (which != 0 && which != 1) || (slab != 0 && slab != 1)) return fail(IRIS_EINVAL, "bad argument");
  CK(cudaSetDevice(E->device));
  const long pc = E->pcomp[slab];
  const int nx = E->p.nx, ny = E->p.ny;
  const long nzs = slab == 0 ? E->nbot : E->ntop;
  void* dev = which == 0 ? E->pml_d[slab] : E->pml_b[slab];
  std::vector<unsigned char> buf((size_t)3 * pc * E->esz);
  if (re) {
    CK(cudaMemcpyAsync(buf.data(), dev, buf.size(), cudaMemcpyDeviceToHost, E->st));
    CK(cudaStreamSynchronize(E->st));
  }
  for (long zr = 0; zr < nzs; ++zr)
    for (int y = 0; y < ny; ++y)
      for (int x = 0; x < nx; ++x)
        for (int c = 0; c < 3; ++c) {
          const long r = c + 3L * (x + (long)nx * (y + (long)ny * zr));
          const long s = c * pc + (zr * ny + y) * (long)nx + x;
          if (E->prec == IRIS_FP64) {
            double* b = (double*)buf.data();
            if (re) { re[r] = b[2 * s]; im[r] = b[2 * s + 1]; }
            else { b[2 * s] = cre[r]; b[2 * s + 1] = cim[r]; }
          } else {
            float* b = (float*)buf.data();
            if (re) { re[r] = b[2 * s]; im[r] = b[2 * s + 1]; }
            else { b[2 * s] = (float)cre[r]; b[2 * s + 1] = (float)cim[r]; }
          }
        }
  if (!re) {
    CK(cudaMemcpyAsync(dev, buf.data(), buf.size(), cudaMemcpyHostToDevice, E->st));
    CK(cudaStreamSynchronize(E->st));
  }
  return IRIS_OK;
}

// Chunked transfer between the host array c (interleaved re, im doubles in
// the host layout of m, planes z_first .. z_first + nplanes - 1) and the
// device arrays dev (get: device to host; else host to device).
static int xfer_c(iris_engine* E, void* dev, const XferMap& m, int z_first, int nplanes, double* c, bool get) {
  const size_t per_plane = (size_t)3 * m.nx * m.ny * sizeof(double2);
  const size_t cap = std::max<size_t>(per_plane, (size_t)64 << 20);
  if (E->stage_bytes < std::min(cap, per_plane * nplanes)) {
    if (E->d_stage) CK(cudaFree(E->d_stage));
    E->d_stage = nullptr;
    E->stage_bytes = std::min(cap, per_plane * nplanes);
    CK(cudaMalloc(&E->d_stage, E->stage_bytes));
  }
  const int chunk = (int)std::max<size_t>(1, E->stage_bytes / per_plane);
  for (int z0 = 0; z0 < nplanes; z0 += chunk) {
    const int nz = std::min(chunk, nplanes - z0);
    const long n = 3L * m.nx * m.ny * nz;
    double* host = c + 2 * (size_t)3 * m.nx * m.ny * z0;
    const unsigned blocks = (unsigned)((n + 255) / 256);
    if (get) {
      if (E->prec == IRIS_FP64)
        k_pack<double><<<blocks, 256, 0, E->st>>>((const double2*)dev, m, z_first + z0, n, (double2*)E->d_stage);
      else
        k_pack<float><<<blocks, 256, 0, E->st>>>((const float2*)dev, m, z_first + z0, n, (double2*)E->d_stage);
      CK(cudaMemcpyAsync(host, E->d_stage, n * sizeof(double2), cudaMemcpyDeviceToHost, E->st));
    } else {
      CK(cudaMemcpyAsync(E->d_stage, host, n * sizeof(double2), cudaMemcpyHostToDevice, E->st));
      if (E->prec == IRIS_FP64)
        k_unpack<double><<<blocks, 256, 0, E->st>>>((double2*)dev, m, z_first + z0, n, (const double2*)E->d_stage);
      else
        k_unpack<float><<<blocks, 256, 0, E->st>>>((float2*)dev, m, z_first + z0, n, (const double2*)E->d_stage);
    }
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(E->st));
  }
  return IRIS_OK;
}

static int field_c(iris_engine* E, int which, double* c, bool get) {
  if (!E || !c || (which != IRIS_E && which != IRIS_H)) return fail(IRIS_EINVAL, "bad argument");
  CK(cudaSetDevice(E->device));
  XferMap m{};
  m.g = E->g;
  m.pc = E->g.comp;
  m.nx = E->p.nx + 2;
  m.ny = E->p.ny + 2;
  return xfer_c(E, which == IRIS_E ? E->e : E->h, m, 0, E->p.nz + 2, c, get);
}

static int pml_c(iris_engine* E, int which, int slab, double* c, bool get) {
  if (!E || !c || (which != 0 && which != 1) || (slab != 0 && slab != 1)) return fail(IRIS_EINVAL, "bad argument");
  CK(cudaSetDevice(E->device));
  XferMap m{};
  m.pc = E->pcomp[slab];
  m.nx = E->p.nx;
  m.ny = E->p.ny;
  m.ox = m.oy = 1;
  m.pml = 1;
  return xfer_c(E, which == 0 ? E->pml_d[slab] : E->pml_b[slab], m, 0, slab == 0 ? E->nbot : E->ntop, c, get);
}

int iris_get_field_c(iris_engine* E, int which, double* c) {
  clear_error();
  return field_c(E, which, c, true);
}

int iris_set_field_c(iris_engine* E, int which, const double* c) {
  clear_error();
  return field_c(E, which, const_cast<double*>(c), false);
}

int iris_get_pml_c(iris_engine* E, int which, int slab, double* c) {
  clear_error();
  return pml_c(E, which, slab, c, true);
}

int iris_set_pml_c(iris_engine* E, int which, int slab, const double* c) {
  clear_error();
  return pml_c(E, which, slab, const_cast<double*>(c), false);
}

int iris_get_pml(iris_engine* E, int which, int slab, double* re, double* im) {
  clear_error();
  if (!re || !im) return fail(IRIS_EINVAL, "null buffer");
  return pml_io(E, which, slab, re, im, nullptr, nullptr);
}

int iris_set_pml(iris_engine* E, int which, int slab, const double* re, const double* im) {
  clear_error();
  if (!re || !im) return fail(IRIS_EINVAL, "null buffer");
  return pml_io(E, which, slab, nullptr, nullptr, re, im);
}

int iris_get_plane(iris_engine* E, int which, int axis, int index, int lo1, int hi1, int lo2, int hi2, double* re,
                   double* im) {
  clear_error();
  if (!E || !re || !im || (which != IRIS_E && which != IRIS_H) || axis < 1 || axis > 3)
    return fail(IRIS_EINVAL, "bad argument");
  const int n[3] = {E->p.nx, E->p.ny, E->p.nz};
  const int ax1 = axis == 1 ? 1 : 0, ax2 = axis == 3 ? 1 : 2;
  if (index < 0 || index > n[axis - 1] + 1 || lo1 < 0 || hi1 > n[ax1] + 1 || lo1 > hi1 || lo2 < 0 ||
      hi2 > n[ax2] + 1 || lo2 > hi2)
    return fail(IRIS_EINVAL, "plane outside the grid (ghost cells 0..n+1 included)");
  CK(cudaSetDevice(E->device));
  const int n1 = hi1 - lo1 + 1, n2 = hi2 - lo2 + 1;
  const long m = 3L * n1 * n2;
  double2* d = nullptr;
  CK(cudaMalloc(&d, sizeof(double2) * m));
  const void* f = which == IRIS_E ? E->e : E->h;
  const unsigned nb = (unsigned)((m + 255) / 256);
  if (E->prec == IRIS_FP64)
    k_plane<double><<<nb, 256, 0, E->st>>>((const double2*)f, E->g, axis, index, lo1, n1, lo2, n2, d);
  else
    k_plane<float><<<nb, 256, 0, E->st>>>((const float2*)f, E->g, axis, index, lo1, n1, lo2, n2, d);
  std::vector<double2> h((size_t)m);
  cudaError_t e1 = cudaMemcpyAsync(h.data(), d, sizeof(double2) * m, cudaMemcpyDeviceToHost, E->st);
  cudaError_t e2 = cudaStreamSynchronize(E->st);
  cudaFree(d);
  if (e1 != cudaSuccess || e2 != cudaSuccess) return fail(IRIS_ECUDA, "plane extraction failed");
  for (long q = 0; q < m; ++q) {
    re[q] = h[q].x;
    im[q] = h[q].y;
  }
  return IRIS_OK;
}

int iris_get_fdata(iris_engine* E, int box, int j, double* re, double* im, long* npts) {
  clear_error();
  if (!E || box < 0 || box > 1 || j < 1 || j > 3) return fail(IRIS_EINVAL, "bad argument");
  CK(cudaSetDevice(E->device));
  if (box >= E->nboxes) box = 0;
  const FaceMap& F = E->fm[box][j - 1];
  const long n = F.active ? 12 * F.nloc : 0;
  if (npts) *npts = n;
  if (!re || n == 0) return IRIS_OK;
  if (!im) return fail(IRIS_EINVAL, "null buffer");
  dft_flush(E);
  if (int rc = fd_materialise(E)) return rc;
  const int nof = E->p.nof;
  // 16 bytes per value: a double2, or in FP32 mode the double-float pairs
  // (re_hi, im_hi, re_lo, im_lo) whose sums are exact in FP64
  const bool df = E->prec != IRIS_FP64;
  std::vector<double2> row((size_t)E->P);
  for (int iw = 0; iw < nof; ++iw) {
    CK(cudaMemcpyAsync(row.data(), (const char*)E->fd + (size_t)iw * E->P * 16, 16 * (size_t)E->P,
                       cudaMemcpyDeviceToHost, E->st));
    CK(cudaStreamSynchronize(E->st));
    for (int side = 0; side < 2; ++side)
      for (int ip = 0; ip < 6; ++ip)
        for (long L = 0; L < F.nloc; ++L) {
          const long q = side * 6 * F.nloc + ip + 6 * L;
          const double2 v = row[F.base[side][ip] + L];
          if (df) {
            float f[4];
            std::memcpy(f, &v, sizeof f);
            re[(size_t)iw * n + q] = (double)f[0] + (double)f[2];
            im[(size_t)iw * n + q] = (double)f[1] + (double)f[3];
          } else {
            re[(size_t)iw * n + q] = v.x;
            im[(size_t)iw * n + q] = v.y;
          }
        }
  }
  return IRIS_OK;
}

int iris_timing(iris_engine* E, int enable) {
  clear_error();
  if (!E) return fail(IRIS_EINVAL, "null engine");
  CK(cudaSetDevice(E->device));
  if (!E->t0) {
    CK(cudaEventCreate(&E->t0));
    CK(cudaEventCreate(&E->t1));
  }
  for (int k = 0; k < IRIS_NKC; ++k) E->ev_used[k] = 0;
  E->timing = enable != 0;
  CK(cudaEventRecord(E->t0, E->st));
  return IRIS_OK;
}

int iris_timing_read(iris_engine* E, double* region_ms, double* kernel_ms, long* launches) {
  clear_error();
  if (!E || !E->t0) return fail(IRIS_EINVAL, "timing was not started");
  CK(cudaSetDevice(E->device));
  CK(cudaEventRecord(E->t1, E->st));
  CK(cudaEventSynchronize(E->t1));
  float ms = 0.f;
  CK(cudaEventElapsedTime(&ms, E->t0, E->t1));
  if (region_ms) *region_ms = ms;
  for (int k = 0; k < IRIS_NKC; ++k) {
    double tot = 0.0;
    for (size_t i = 0; i < E->ev_used[k]; ++i) {
      float x = 0.f;
      CK(cudaEventElapsedTime(&x, E->ev[k][i].first, E->ev[k][i].second));
      tot += x;
    }
    if (kernel_ms) kernel_ms[k] = tot;
    if (launches) launches[k] = (long)E->ev_used[k];
  }
  E->timing = false;
  return stream_status(E);
}

int iris_info(const iris_engine* E, long* info) {
  if (!E || !info) return fail(IRIS_EINVAL, "bad argument");
  info[0] = E->P;
  info[1] = E->K;
  info[2] = (long)E->esz;
  info[3] = E->g.comp;
  info[4] = E->eps_complex ? 1 : 0;
  info[5] = E->nboxes;
  info[6] = E->nslot;
  return IRIS_OK;
}

int iris_bounds_check(unsigned long long* first) {
  clear_error();
  if (!first) return fail(IRIS_EINVAL, "bad argument");
  const unsigned long long r[3] = {bc_take_module(), bc_take_batch(), bc_take_adjoint()};
  *first = 0;
  for (unsigned long long v : r)
    if (v && !*first) *first = v;
#ifdef IRIS_BOUNDS_CHECK
  return 1;
#else
  return 0;
#endif
}

int iris_dft_commit(iris_engine* E) {
  iris::NvtxRange nvtx_("iris_dft_commit");
  clear_error();
  if (!E) return fail(IRIS_EINVAL, "null engine");
  CK(cudaSetDevice(E->device));
  dft_flush(E);
  CK(cudaGetLastError());
  return IRIS_OK;
}

int iris_apply(iris_engine* E, int op, int arg) {
  clear_error();
  if (!E) return fail(IRIS_EINVAL, "null engine");
  CK(cudaSetDevice(E->device));
  const bool d = E->prec == IRIS_FP64;
  switch (op) {
    case IRIS_OP_E: d ? launch_e<double>(E) : launch_e<float>(E); break;
    case IRIS_OP_H: d ? launch_h<double>(E) : launch_h<float>(E); break;
    case IRIS_OP_TFSF: d ? launch_tfsf<double>(E, arg) : launch_tfsf<float>(E, arg); break;
    case IRIS_OP_DFT:
      dft_flush(E);
      d ? dft_sample<double>(E, arg) : dft_sample<float>(E, arg);
      dft_flush(E);
      break;
    case IRIS_OP_WAIT_CHECK:
      if (arg < 0 || arg > 30) return fail(IRIS_EINVAL, "wait check: arg must be 0..30");
      k_wait_check<<<1, 32, 0, E->st>>>(E->d_err, arg);
      break;
    case IRIS_OP_BARRIER_CHECK: {
      if (arg < 0 || arg > 30) return fail(IRIS_EINVAL, "barrier check: arg must be 0..30");
      if (!E->persist) return fail(IRIS_EINVAL, "barrier check: the engine does not step with the persistent kernel");
      CK(cudaMemsetAsync(E->d_bar, 0, sizeof(GridBar), E->st));
      GridBar* bar = (GridBar*)E->d_bar;
      int* err = E->d_err;
      void* args[] = {&bar, &err, &arg};
      CK(cudaLaunchCooperativeKernel((const void*)k_barrier_check, dim3(2), dim3(32), args, 0, E->st));
      break;
    }
    default: return fail(IRIS_EINVAL, "unknown operator");
  }
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(E->st));
  return stream_status(E);
}

}  // extern "C"

extern "C" const char* iris_last_error(void) { return iris::g_last_error.c_str(); }

// ---------------------------------------------------------------------------
// Allocation-free DFT block accumulation.
//
// The twiddle table that k_dft_fp32 reads lives in this fixed device array
// instead of memory the engine allocates: IRIS_NOALLOC_MAX_TWIDDLES float2
// values (512 KiB), present on every GPU that loads the library until the
// process exits.  Host code cannot use the symbol itself as a device pointer,
// so the first call on each device looks its address up with
// cudaGetSymbolAddress (with that device current) and caches it.  All calls
// share the array: each call overwrites the nk*nof entries it uses, so nothing
// has to be cleared, and two calls whose kernels overlap on the GPU race on it.
static __device__ __align__(256) float2 g_noalloc_twiddles[IRIS_NOALLOC_MAX_TWIDDLES];

namespace {
constexpr int kNoallocMaxDevices = 64;
std::mutex g_noalloc_mu;
void* g_noalloc_addr[kNoallocMaxDevices] = {};
}  // namespace

extern "C" int iris_dft_block_noalloc(const void* samples, int nk, long npts, int t0, int t_step, const double* fw,
                                      int nof, double dt, void* fdata, void* stream) {
  clear_error();
  // every argument check comes before the first CUDA call: a refused call
  // touches no device
  if (!samples || !fw || !fdata) return fail(IRIS_EINVAL, "iris_dft_block_noalloc: null device pointer");
  if (nk < 1 || npts < 1 || nof < 1) return fail(IRIS_EINVAL, "iris_dft_block_noalloc: nk, npts and nof must be >= 1");
  if ((uintptr_t)samples % 8 || (uintptr_t)fw % 8 || (uintptr_t)fdata % 16)
    return fail(IRIS_EINVAL,
                "iris_dft_block_noalloc: samples and fw must be 8-byte aligned, fdata 16-byte aligned");
  if ((long)nk * nof > IRIS_NOALLOC_MAX_TWIDDLES)
    return fail(IRIS_EINVAL, "iris_dft_block_noalloc: nk*nof = " + std::to_string((long)nk * nof) +
                                 " exceeds the static scratch of " + std::to_string(IRIS_NOALLOC_MAX_TWIDDLES) +
                                 " twiddles; split the block");
  const int nwc = (nof + DFT_TW - 1) / DFT_TW;
  const long nblk = (npts + DFT_TP - 1) / DFT_TP;
  if (nblk * nwc > 0x7fffffffL) return fail(IRIS_EINVAL, "iris_dft_block_noalloc: npts too large for one launch");
  int dev = 0;
  CK(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kNoallocMaxDevices) return fail(IRIS_EINVAL, "iris_dft_block_noalloc: device ordinal >= 64");
  // an error left by earlier work on this thread is reported as such, not
  // taken for this call's, and nothing is launched
  const cudaError_t prior = cudaGetLastError();
  if (prior != cudaSuccess)
    return fail(IRIS_ECUDA, std::string("iris_dft_block_noalloc: a CUDA error from before this call was pending: ") +
                                cudaGetErrorString(prior));
  void* wt = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_addr[dev]) {
      void* a = nullptr;
      const cudaError_t e = cudaGetSymbolAddress(&a, g_noalloc_twiddles);
      if (e != cudaSuccess)
        return fail(IRIS_ECUDA, std::string("iris_dft_block_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
      g_noalloc_addr[dev] = a;
    }
    wt = g_noalloc_addr[dev];
  }
  cudaStream_t st = (cudaStream_t)stream;
  const int nt = nk * nof;
  k_twiddle<<<(nt + 255) / 256, 256, 0, st>>>(nullptr, t0, t_step, nk, fw, nof, dt, (float2*)wt);
  k_dft_fp32<double2><<<(unsigned)(nblk * nwc), DFT_THREADS, 0, st>>>((const float2*)samples, npts, nk, (const float2*)wt, nof,
                                                           nwc, (double2*)fdata);
  CK(cudaGetLastError());
  return IRIS_OK;
}
