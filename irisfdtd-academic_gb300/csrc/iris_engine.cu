// GB300 (sm_103a) FDTD engine: device state, kernels and the C ABI that
// replaces the per-step operators of IrisFDTD-Academic's driver loop
// (code/driver.f90:338-451).
//
// Data layout in HBM
//   * E and H: three component arrays each, complex (double2 in FP64 mode,
//     float2 in FP32 mode), x fastest, ghost planes 0 and n+1 on every axis,
//     rows padded so that x = 1 starts on a 128-byte boundary.  Updated in
//     place: the leapfrog update of a cell reads only its own old value, so
//     the reference's cur/prev pointer swap (code/driver.f90:358-384) needs no
//     second copy.
//   * UPML auxiliaries D and B exist for the two z slabs only, also updated
//     in place.
//   * Structure inverse permittivity over z in [hi, hf] (real when the
//     material is lossless, complex otherwise).
//   * DFT: a ring of K sample slots [K][P] gathered from the box faces after
//     each sampled step, accumulated into fdata [nof][P] (complex double)
//     one block of samples at a time.
//
// Arithmetic: the FP64 mode uses __dmul_rn/__dadd_rn (never contracted to
// FMA) so the stencil rounds exactly like the reference build; the FP32 mode
// lets the compiler contract.
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

#include "iris_internal.h"

namespace iris {
namespace {

// ---------------------------------------------------------------------------
// device arithmetic

template <typename T> struct V2;
template <> struct V2<double> { using t = double2; };
template <> struct V2<float> { using t = float2; };

template <typename T> __device__ __forceinline__ T mul_(T a, T b);
template <typename T> __device__ __forceinline__ T add_(T a, T b);
template <typename T> __device__ __forceinline__ T sub_(T a, T b);
template <> __device__ __forceinline__ double mul_<double>(double a, double b) { return __dmul_rn(a, b); }
template <> __device__ __forceinline__ double add_<double>(double a, double b) { return __dadd_rn(a, b); }
template <> __device__ __forceinline__ double sub_<double>(double a, double b) { return __dsub_rn(a, b); }
template <> __device__ __forceinline__ float mul_<float>(float a, float b) { return a * b; }
template <> __device__ __forceinline__ float add_<float>(float a, float b) { return a + b; }
template <> __device__ __forceinline__ float sub_<float>(float a, float b) { return a - b; }

template <typename T> struct cx { T re, im; };

template <typename T> __device__ __forceinline__ cx<T> cadd(cx<T> a, cx<T> b) { return {add_(a.re, b.re), add_(a.im, b.im)}; }
template <typename T> __device__ __forceinline__ cx<T> csub(cx<T> a, cx<T> b) { return {sub_(a.re, b.re), sub_(a.im, b.im)}; }
template <typename T> __device__ __forceinline__ cx<T> rmul(T r, cx<T> a) { return {mul_(r, a.re), mul_(r, a.im)}; }
template <typename T> __device__ __forceinline__ cx<T> cmul(cx<T> a, cx<T> b) {
  return {sub_(mul_(a.re, b.re), mul_(a.im, b.im)), add_(mul_(a.re, b.im), mul_(a.im, b.re))};
}
template <typename T> __device__ __forceinline__ cx<T> ld(const typename V2<T>::t* p) {
  typename V2<T>::t v = *p;
  return {v.x, v.y};
}
template <typename T> __device__ __forceinline__ void st(typename V2<T>::t* p, cx<T> a) {
  typename V2<T>::t v;
  v.x = a.re;
  v.y = a.im;
  *p = v;
}

// ---------------------------------------------------------------------------
// geometry of a ghost-padded field component

struct Geo {
  int nx, ny, nz;
  long pitch, plane, comp;  // in elements
  int xo;                   // storage index of x is x + xo
  __host__ __device__ __forceinline__ long at(int x, int y, int z) const {
    return (long)z * plane + (long)y * pitch + (long)(x + xo);
  }
};

// UPML coefficient row (24 per PML z-plane), see make_coef()
enum { CD_A = 0, CD_B = 3, CE_A = 6, CE_B = 9, C_FP = 12, C_FM = 15, CB_B = 18, CH_B = 21, NCOEF = 24 };

template <typename T> struct FieldArgs {
  typename V2<T>::t* e;  // component 0; components 1,2 at +comp, +2 comp
  typename V2<T>::t* h;
  Geo g;
  typename V2<T>::t* pml_d[2];
  typename V2<T>::t* pml_b[2];
  long pcomp[2];
  const T* coef;
  int pmlzi, pmlzf, hi, hf;
  const typename V2<T>::t* eps_c;  // complex structure material or null
  const T* eps_r;                  // real structure material or null
  T m1, m3, eps0sq, dtcq2;
  cx<T> pxp, pyp, pzp, pxm, pym, pzm;  // Bloch phases exp(+-i ak)
};

// New E of interior cell (x, y, z) from the curl of the old H (c) and the
// old E (e, replaced): the material and UPML part of e_fdtd
// (code/fdtd.f90:57-153) and UPML_Array_e (code/boundary_II.f90:60-138).
// Per z the reference's region order decides: the UPML slabs overwrite
// whatever e_fdtd wrote there.  The UPML auxiliary is read from a.pml_d and,
// when dnew is given, its new value written there (dnew == a.pml_d updates in
// place).  With EPV the caller supplies the real structure eps_inv of the
// cell (ep) instead of it being read from a.eps_r.  MASK selects the
// components computed (bit k: E_{k+1}).  UPML = false: the caller knows the
// cell lies outside the UPML slabs (the slab code is not compiled in).
template <typename T, bool CEPS, int MASK = 7, bool EPV = false, bool UPML = true>
__device__ __forceinline__ void e_apply(const FieldArgs<T>& a, typename V2<T>::t* const* dnew, int x, int y, int z,
                                        const cx<T> c[3], cx<T> e[3], T ep = T(0)) {
  using V = typename V2<T>::t;
  const Geo& g = a.g;
  if (UPML && (z <= a.pmlzi || z >= a.pmlzf)) {
    const int slab = z <= a.pmlzi ? 0 : 1;
    const int zr = slab == 0 ? z - 1 : z - a.pmlzf;
    const int row = slab == 0 ? z - 1 : a.pmlzi + z - a.pmlzf;
    const T* cf = a.coef + NCOEF * row;
    const long pi = ((long)zr * g.ny + (y - 1)) * (long)g.nx + (x - 1);
    const V* D = a.pml_d[slab];
    const long pc = a.pcomp[slab];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      if (!(MASK & (1 << k))) continue;
      const cx<T> ck = rmul(a.eps0sq, c[k]);
      const cx<T> dold = ld<T>(D + k * pc + pi);
      const cx<T> dn = cadd(rmul(cf[CD_A + k], dold), rmul(cf[CD_B + k], ck));
      if (dnew) st<T>(dnew[slab] + k * pc + pi, dn);
      e[k] = cadd(rmul(cf[CE_A + k], e[k]), rmul(cf[CE_B + k], csub(rmul(cf[C_FP + k], dn), rmul(cf[C_FM + k], dold))));
    }
  } else if (z >= a.hi && z <= a.hf) {
    const long ie = (long)(z - a.hi) * g.plane + (long)y * g.pitch + (long)(x + g.xo);
    if (CEPS) {
      const cx<T> epc = ld<T>(a.eps_c + ie);
#pragma unroll
      for (int k = 0; k < 3; ++k)
        if (MASK & (1 << k)) e[k] = cadd(e[k], cmul(epc, c[k]));
    } else {
      const T epr = EPV ? ep : a.eps_r[ie];
#pragma unroll
      for (int k = 0; k < 3; ++k)
        if (MASK & (1 << k)) e[k] = cadd(e[k], rmul(epr, c[k]));
    }
  } else {
    const T m = z < a.hi ? a.m1 : a.m3;
#pragma unroll
    for (int k = 0; k < 3; ++k)
      if (MASK & (1 << k)) e[k] = cadd(e[k], rmul(m, c[k]));
  }
}

// The E update of one cell given its own old H (h), the old H one plane
// below (hzm, components 1 and 2) and its old E (e, replaced by the new E);
// the x-1 and y-1 neighbours are loaded here.  MASK selects the components
// computed (bit k: E_{k+1}); loads only the others need are never issued.
template <typename T, bool CEPS, int MASK = 7, bool UPML = true>
__device__ __forceinline__ void e_update(const FieldArgs<T>& a, typename V2<T>::t* const* dnew, int x, int y, int z,
                                         const cx<T> h[3], const cx<T> hzm[3], cx<T> e[3]) {
  using V = typename V2<T>::t;
  const Geo& g = a.g;
  const long i = g.at(x, y, z);
  const V* H1 = a.h;
  const V* H2 = a.h + g.comp;
  const V* H3 = a.h + 2 * g.comp;
  cx<T> c[3];
  if (MASK & 1) c[0] = cadd(csub(csub(h[2], ld<T>(H3 + i - g.pitch)), h[1]), hzm[1]);
  if (MASK & 2) c[1] = cadd(csub(csub(h[0], hzm[0]), h[2]), ld<T>(H3 + i - 1));
  if (MASK & 4) c[2] = cadd(csub(csub(h[1], ld<T>(H2 + i - 1)), h[0]), ld<T>(H1 + i - g.pitch));
  e_apply<T, CEPS, MASK, false, UPML>(a, dnew, x, y, z, c, e);
}

// New E of interior cell (x, y, z) from the old E and H in memory: e_fdtd
// (code/fdtd.f90:57-153) and UPML_Array_e (code/boundary_II.f90:60-138).
template <typename T, bool CEPS, int MASK = 7, bool UPML = true>
__device__ __forceinline__ void e_cell(const FieldArgs<T>& a, typename V2<T>::t* const* dnew, int x, int y, int z,
                                       cx<T> e[3]) {
  const Geo& g = a.g;
  const long i = g.at(x, y, z);
  cx<T> h[3], hzm[3];
  // own H: c1 uses H3, H2; c2 uses H1, H3; c3 uses H2, H1
  if (MASK & 6) h[0] = ld<T>(a.h + i);
  if (MASK & 5) h[1] = ld<T>(a.h + g.comp + i);
  if (MASK & 3) h[2] = ld<T>(a.h + 2 * g.comp + i);
  if (MASK & 2) hzm[0] = ld<T>(a.h + i - g.plane);
  if (MASK & 1) hzm[1] = ld<T>(a.h + g.comp + i - g.plane);
#pragma unroll
  for (int k = 0; k < 3; ++k)
    if (MASK & (1 << k)) e[k] = ld<T>(a.e + k * g.comp + i);
  e_update<T, CEPS, MASK, UPML>(a, dnew, x, y, z, h, hzm, e);
}

// New H of interior cell (x, y, z): h_fdtd (code/fdtd.f90:157-248) and
// UPML_Array_h (code/boundary_II.f90:142-220), from the new E of the cell (ev)
// and of its +x, +y, +z neighbours (xp: components 2,3; yp: 1,3; zp: 1,2),
// the old H read from a.h, the UPML auxiliary B updated in place.  UPML =
// false: the cell lies outside the UPML slabs.
template <typename T, bool UPML = true>
__device__ __forceinline__ void h_update(const FieldArgs<T>& a, int x, int y, int z, const cx<T> ev[3],
                                         const cx<T> xp[3], const cx<T> yp[3], const cx<T> zp[3], cx<T> h[3]) {
  using V = typename V2<T>::t;
  const Geo& g = a.g;
  cx<T> c[3];
  c[0] = cadd(csub(csub(yp[2], ev[2]), zp[1]), ev[1]);
  c[1] = cadd(csub(csub(zp[0], ev[0]), xp[2]), ev[2]);
  c[2] = cadd(csub(csub(xp[1], ev[1]), yp[0]), ev[0]);
  if (UPML && (z <= a.pmlzi || z >= a.pmlzf)) {
    const int slab = z <= a.pmlzi ? 0 : 1;
    const int zr = slab == 0 ? z - 1 : z - a.pmlzf;
    const int row = slab == 0 ? z - 1 : a.pmlzi + z - a.pmlzf;
    const T* cf = a.coef + NCOEF * row;
    const long pi = ((long)zr * g.ny + (y - 1)) * (long)g.nx + (x - 1);
    V* B = a.pml_b[slab];
    const long pc = a.pcomp[slab];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const cx<T> bold = ld<T>(B + k * pc + pi);
      const cx<T> bn = csub(rmul(cf[CD_A + k], bold), rmul(cf[CB_B + k], c[k]));
      st<T>(B + k * pc + pi, bn);
      h[k] = cadd(rmul(cf[CE_A + k], h[k]), rmul(cf[CH_B + k], csub(rmul(cf[C_FP + k], bn), rmul(cf[C_FM + k], bold))));
    }
  } else {
#pragma unroll
    for (int k = 0; k < 3; ++k) h[k] = csub(h[k], rmul(a.dtcq2, c[k]));
  }
}

// h_update with the old H of the cell loaded from a.h.
template <typename T, bool UPML = true>
__device__ __forceinline__ void h_cell(const FieldArgs<T>& a, int x, int y, int z, const cx<T> ev[3],
                                       const cx<T> xp[3], const cx<T> yp[3], const cx<T> zp[3], cx<T> h[3]) {
  const long i = a.g.at(x, y, z);
#pragma unroll
  for (int k = 0; k < 3; ++k) h[k] = ld<T>(a.h + k * a.g.comp + i);
  h_update<T, UPML>(a, x, y, z, ev, xp, yp, zp, h);
}

// Split E pass of one cell: e_cell in place + bc_{x,y,z}max_bloch
// (code/boundary.f90:193-216,257-284,321-348) for the E ghosts.
template <typename T, bool CEPS, bool UPML = true>
__device__ __forceinline__ void e_split_cell(const FieldArgs<T>& a, int x, int y, int z) {
  using V = typename V2<T>::t;
  const Geo& g = a.g;
  const long i = g.at(x, y, z);
  V* E[3] = {a.e, a.e + g.comp, a.e + 2 * g.comp};
  cx<T> e[3];
  e_cell<T, CEPS, 7, UPML>(a, a.pml_d, x, y, z, e);
#pragma unroll
  for (int k = 0; k < 3; ++k) st<T>(E[k] + i, e[k]);
  if (x == 1) {
    const long j = g.at(g.nx + 1, y, z);
#pragma unroll
    for (int k = 0; k < 3; ++k) st<T>(E[k] + j, cmul(a.pxp, e[k]));
  }
  if (y == 1) {
    const long j = g.at(x, g.ny + 1, z);
#pragma unroll
    for (int k = 0; k < 3; ++k) st<T>(E[k] + j, cmul(a.pyp, e[k]));
  }
  if (z == 1) {
    const long j = g.at(x, y, g.nz + 1);
#pragma unroll
    for (int k = 0; k < 3; ++k) st<T>(E[k] + j, cmul(a.pzp, e[k]));
  }
}

template <typename T, bool CEPS>
__global__ void __launch_bounds__(256) k_update_e(FieldArgs<T> a) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int y = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int z = blockIdx.z * blockDim.z + threadIdx.z + 1;
  if (x > a.g.nx || y > a.g.ny || z > a.g.nz) return;
  e_split_cell<T, CEPS>(a, x, y, z);
}

// Split H pass of one cell: h_cell in place + bc_{x,y,z}min_bloch
// (code/boundary.f90:163-187,224-251,288-315) for the H ghosts and the E
// ghosts at 0.  The ghosts at nx+1/ny+1/nz+1 of H are never read by any
// operator and are not maintained.
template <typename T, bool UPML = true>
__device__ __forceinline__ void h_split_cell(const FieldArgs<T>& a, int x, int y, int z) {
  using V = typename V2<T>::t;
  const Geo& g = a.g;
  const long i = g.at(x, y, z);
  V* Ec[3] = {a.e, a.e + g.comp, a.e + 2 * g.comp};
  V* H[3] = {a.h, a.h + g.comp, a.h + 2 * g.comp};
  cx<T> ev[3], xp[3], yp[3], zp[3], h[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) ev[k] = ld<T>(Ec[k] + i);
  xp[1] = ld<T>(Ec[1] + i + 1);
  xp[2] = ld<T>(Ec[2] + i + 1);
  yp[0] = ld<T>(Ec[0] + i + g.pitch);
  yp[2] = ld<T>(Ec[2] + i + g.pitch);
  zp[0] = ld<T>(Ec[0] + i + g.plane);
  zp[1] = ld<T>(Ec[1] + i + g.plane);
  h_cell<T, UPML>(a, x, y, z, ev, xp, yp, zp, h);
#pragma unroll
  for (int k = 0; k < 3; ++k) st<T>(H[k] + i, h[k]);
  if (x == g.nx) {
    const long j = g.at(0, y, z);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      st<T>(Ec[k] + j, cmul(a.pxm, ev[k]));
      st<T>(H[k] + j, cmul(a.pxm, h[k]));
    }
  }
  if (y == g.ny) {
    const long j = g.at(x, 0, z);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      st<T>(Ec[k] + j, cmul(a.pym, ev[k]));
      st<T>(H[k] + j, cmul(a.pym, h[k]));
    }
  }
  if (z == g.nz) {
    const long j = g.at(x, y, 0);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      st<T>(Ec[k] + j, cmul(a.pzm, ev[k]));
      st<T>(H[k] + j, cmul(a.pzm, h[k]));
    }
  }
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

__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

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

// ---------------------------------------------------------------------------
// TF/SF source: tfsf_gauss (code/tfsf.f90:231-355) or tfsf_plane_wave
// (code/tfsf.f90:359-517) evaluated in FP64 at the two planes the update
// reads, then tfsf_update_3DArray (code/tfsf.f90:76-153) or
// tfsf_update_2DArray (code/tfsf.f90:163-227) over the reference's ranges,
// ghosts included.  The incident field is y-independent, so each thread
// evaluates it once for its ix and walks a chunk of iy.

struct SrcArgs {
  int variant;  // 0 none, 1 update_3DArray, 2 update_2DArray
  int i_pol, plane_wave, cosine;
  int nx, ny, iz_min;
  int ixo, izo_i;  // izo_i: the INTEGER izo of tfsf_plane_wave
  double izo;      // the REAL izo of tfsf_gauss (zopump)
  double Q, c0dt, ko, Dk, ux, uz;
  double sign_kz;  // +1 source in the cover, -1 in the substrate
  double sq_eps;   // sqrt(eps of the source medium)
  double sqs;      // sqrt(eps)*sign_kz
  double uzs;      // u_z*sign_kz
  double amp;      // Epump*Q
  double hcoef;    // Epump*Q*(dt*c0/Q)
  double eps_in1, eps_src, dtcq2, s1, tincr, tdecay;
};


__device__ __forceinline__ double dm(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double da(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double ds(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dq(double a, double b) { return __ddiv_rn(a, b); }

// Incident field at (ix, iz), step it.  i_pol = 2: ta = tf1 (E_x), tb = tf5
// (H_y, scaled by dt*c0/Q); i_pol = 1: ta = tf2 (E_y), tb = tf4 (H_x).  The
// expressions keep the reference's association (code/tfsf.f90:306-347 and
// :430-508), with exact shortcuts only where a factor is (1,0) or +-1.
__device__ void incident(const SrcArgs& s, int ix, int iz, int it, cx<double>& ta, cx<double>& tb) {
  double cs, sn, env;
  const double t = dm(s.c0dt, (double)it);  // c0*dt*(it-ito), ito = 0
  const bool gauss = s.plane_wave == 1;
  if (gauss) {
    const double A = da(dm(dm(s.Q, (double)(ix - s.ixo)), s.ux), dm(dm(s.Q, ds((double)iz, s.izo)), s.uz));
    const double kzz = dm(s.ko, ds(dm(s.sqs, A), t));
    const double arg = dq(ds(A, dq(t, s.sq_eps)), s.Dk);
    env = exp(-dm(arg, arg));
    sincos(kzz, &sn, &cs);
  } else {
    const double A = da(dm(dm(s.Q, (double)(ix - s.ixo)), s.ux), dm(dm(s.Q, (double)(iz - s.izo_i)), s.uz));
    const double kzz = dm(s.ko, ds(A, dq(t, s.s1)));
    const double d = dm(s.Q, fabs((double)(iz - s.izo_i)));
    const double ton = dm(s.c0dt, ds((double)it, s.tincr));
    const double toff = dm(s.c0dt, ds((double)it, s.tdecay));
    if (ton <= d) env = exp(dq(-ds(d, ton), s.Dk));
    else if (toff >= d) env = exp(dq(ds(d, toff), s.Dk));
    else env = 1.0;
    sincos(kzz, &sn, &cs);
  }
  const double sg = gauss ? s.sign_kz : 1.0;
  // sign*(1,0)*exp(i kzz)*env  ->  (env*(sign*c), env*(sign*s))
  const cx<double> w{dm(env, dm(sg, cs)), dm(env, dm(sg, sn))};
  const cx<double> w1{dm(env, cs), dm(env, sn)};  // (1,0)*exp(i kzz)*env
  if (s.i_pol == 2) {
    const cx<double> ex{dm(s.uz, w.re), dm(s.uz, w.im)};
    const cx<double> ez{-dm(s.ux, w1.re), -dm(s.ux, w1.im)};
    cx<double> hy;
    if (gauss) hy = {ds(dm(s.uzs, ex.re), dm(s.ux, ez.re)), ds(dm(s.uzs, ex.im), dm(s.ux, ez.im))};
    else hy = {dm(s.s1, ds(dm(s.uz, ex.re), dm(s.ux, ez.re))), dm(s.s1, ds(dm(s.uz, ex.im), dm(s.ux, ez.im)))};
    cx<double> exo = ex;
    if (s.cosine == 1) {
      exo.im = 0.0;
      hy.im = 0.0;
    }
    ta = {dm(s.amp, exo.re), dm(s.amp, exo.im)};
    tb = {dm(s.hcoef, hy.re), dm(s.hcoef, hy.im)};
  } else if (s.i_pol == 1) {
    const cx<double> hx{-dm(s.uz, w.re), -dm(s.uz, w.im)};
    const cx<double> hz{dm(s.ux, w1.re), dm(s.ux, w1.im)};
    cx<double> ey;
    if (gauss) ey = {ds(dm(s.ux, hz.re), dm(s.uzs, hx.re)), ds(dm(s.ux, hz.im), dm(s.uzs, hx.im))};
    else ey = {dm(s.s1, ds(dm(s.ux, hz.re), dm(s.uz, hx.re))), dm(s.s1, ds(dm(s.ux, hz.im), dm(s.uz, hx.im)))};
    cx<double> hxo = hx;
    if (s.cosine == 1) {
      ey.im = 0.0;
      hxo.im = 0.0;
    }
    ta = {dm(s.amp, ey.re), dm(s.amp, ey.im)};
    tb = {dm(s.hcoef, hxo.re), dm(s.hcoef, hxo.im)};
  } else {
    ta = {0.0, 0.0};
    tb = {0.0, 0.0};
  }
}

// Add (sgn=+1) or subtract an FP64 correction to a stored field value.
template <typename T> __device__ __forceinline__ void corr(typename V2<T>::t* p, cx<double> v, int sgn);
template <> __device__ __forceinline__ void corr<double>(double2* p, cx<double> v, int sgn) {
  double2 a = *p;
  if (sgn > 0) { a.x = da(a.x, v.re); a.y = da(a.y, v.im); }
  else { a.x = ds(a.x, v.re); a.y = ds(a.y, v.im); }
  *p = a;
}
template <> __device__ __forceinline__ void corr<float>(float2* p, cx<double> v, int sgn) {
  float2 a = *p;
  if (sgn > 0) { a.x = (float)((double)a.x + v.re); a.y = (float)((double)a.y + v.im); }
  else { a.x = (float)((double)a.x - v.re); a.y = (float)((double)a.y - v.im); }
  *p = a;
}

constexpr int TFSF_YCH = 16;

// Incident field at ix and the corrections of the rows iy in [y0, y1].
template <typename T>
__device__ __forceinline__ void tfsf_column(typename V2<T>::t* e, typename V2<T>::t* h, const Geo& g,
                                            const SrcArgs& s, int it, int ix, int y0, int y1) {
  const int zm = s.iz_min;
  cx<double> ta, tb, vE, vH;
  typename V2<T>::t *pe, *ph;
  int sE, sH, exE, exH, eyE, eyH;  // ix limit and iy limit per update
  if (s.variant == 1) {
    cx<double> a0, b0, a1, b1;
    incident(s, ix, zm - 1, it, a0, b0);  // tfsf_data(:, ix, iy, iz_min-1)
    incident(s, ix, zm, it, a1, b1);      // tfsf_data(:, ix, iy, iz_min)
    vE = {dm(s.eps_in1, b0.re), dm(s.eps_in1, b0.im)};
    vH = {dm(s.dtcq2, a1.re), dm(s.dtcq2, a1.im)};
    if (s.i_pol == 2) {
      // E_x(iz_min) += eps_in(1)*tf5(iz_min-1): ix in [0,nx], iy in [0,ny+1]
      // H_y(iz_min-1) += dtcq2*tf1(iz_min):      ix in [0,nx], iy in [0,ny+1]
      pe = e;
      ph = h + g.comp;
      sE = +1; sH = +1;
      exE = s.nx; exH = s.nx; eyE = s.ny + 1; eyH = s.ny + 1;
    } else {
      // E_y(iz_min) -= eps_in(1)*tf4(iz_min-1): ix in [0,nx+1], iy in [0,ny]
      // H_x(iz_min-1) -= dtcq2*tf2(iz_min):      ix in [0,nx+1], iy in [0,ny]
      pe = e + g.comp;
      ph = h;
      sE = -1; sH = -1;
      exE = s.nx + 1; exH = s.nx + 1; eyE = s.ny; eyH = s.ny;
    }
    for (int iy = y0; iy <= y1; ++iy) {
      if (ix <= exE && iy <= eyE) corr<T>(pe + g.at(ix, iy, zm), vE, sE);
      if (ix <= exH && iy <= eyH) corr<T>(ph + g.at(ix, iy, zm - 1), vH, sH);
    }
  } else if (s.variant == 2) {
    // E_x(iz_min) += tf5(iz_min)/eps ; H_y(iz_min) += dtcq2*tf1(iz_min)
    incident(s, ix, zm, it, ta, tb);
    vE = {dq(tb.re, s.eps_src), dq(tb.im, s.eps_src)};
    vH = {dm(s.dtcq2, ta.re), dm(s.dtcq2, ta.im)};
    for (int iy = y0; iy <= y1; ++iy) {
      corr<T>(e + g.at(ix, iy, zm), vE, +1);
      corr<T>(h + g.comp + g.at(ix, iy, zm), vH, +1);
    }
  }
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

// ---------------------------------------------------------------------------
// On-the-fly DFT (code/dataprocess.f90:109-209)

// One contiguous run of sample points: one component on one face of a box,
// locations in the reference's order (code/dataprocess.f90:813-900).
struct Seg {
  long src;    // storage index of the first location
  long su, sv; // storage strides of the two in-face axes
  int nu, nv;  // extents (u fastest)
  int field;   // 0..2 E components, 3..5 H components
  int pad;
  long p0;     // first sample index
};

template <typename T>
__global__ void __launch_bounds__(256) k_dft_gather(const typename V2<T>::t* __restrict__ e,
                                                    const typename V2<T>::t* __restrict__ h, long comp,
                                                    const Seg* __restrict__ segs, typename V2<T>::t* __restrict__ slot,
                                                    int* tk, int islot, int t, const int* tp) {
  if (blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0) tk[islot] = tp ? *tp + t : t;
  const Seg sg = segs[blockIdx.y];
  const long L = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const long n = (long)sg.nu * sg.nv;
  if (L >= n) return;
  const int u = (int)(L % sg.nu), v = (int)(L / sg.nu);
  const typename V2<T>::t* src = sg.field < 3 ? e + sg.field * comp : h + (sg.field - 3) * comp;
  slot[sg.p0 + L] = src[sg.src + (long)u * sg.su + (long)v * sg.sv];
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
// the block of nk samples, then one FP64 add per (p, iw) into fdata.
// CTA tile: 128 points x 32 frequencies, 128 threads (three CTAs per SM, so one
// CTA's staging overlaps the others' FMAs).  Lane l owns points l + 32 i
// (i < 4), warp w owns frequencies 8 w + j (j < 8), so each thread keeps a
// 4 x 8 complex register tile and every k costs 8 shared loads for 128 FMAs.
// Samples and twiddles are staged through shared memory 32 k at a time.  The
// 1-D grid runs the frequency chunks of one point tile back to back so the
// tile's samples are read from HBM once and from L2 after that.
constexpr int DFT_TP = 128, DFT_TW = 32, DFT_KC = 32, DFT_THREADS = 128;
__global__ void __launch_bounds__(DFT_THREADS) k_dft_fp32(const float2* __restrict__ S, long P, int nk,
                                                  const float2* __restrict__ Wt, int nof, int nwc,
                                                  double2* __restrict__ fd) {
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
      double2* q = fd + (long)w * P + p;
      double2 f = *q;
      f.x += (double)ar[i][j];
      f.y += (double)ai[i][j];
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
// A CTA owns TC_M = 128 points (the 128 TMEM lanes) and a group of up to
// TC_NW = 128 frequencies (256 FP32 TMEM columns).  K is walked in chunks of
// TC_KC = 16 (8 samples) through two shared-memory stages: the CTA's four
// warps split the chunk's samples into the hi/lo A operands (K-major core
// matrices, no swizzle) while the previous chunk's twelve MMAs run; the B
// operands, identical for every CTA, are prepared once per block in global
// memory in the same layout by k_twiddle_tc and bulk-copied (TMA) per chunk.
// One elected thread issues the MMAs and commits them to an mbarrier; the
// epilogue reads the accumulators back with tcgen05.ld and adds them to
// fdata in FP64, one coalesced double2 row per frequency.  Every wait is
// bounded; a CTA that gives up records it in err, still waits (bounded) for
// its MMAs, frees its TMEM and exits.

constexpr int TC_M = 128, TC_NW = 128, TC_KC = 16, TC_THREADS = 256;
constexpr int TC_NMAX = 2 * TC_NW;                       // TMEM columns per CTA
constexpr int TC_BROWS = TC_NMAX;                        // B rows per chunk buffer
constexpr size_t TC_A_BYTES = (size_t)TC_M * TC_KC * 4;  // one of A hi / A lo
constexpr size_t TC_B_BYTES = (size_t)TC_BROWS * TC_KC * 4;
constexpr size_t TC_R_BYTES = (size_t)(TC_KC / 2) * TC_M * 8;  // raw samples of one chunk
constexpr size_t TC_STAGE = 2 * TC_A_BYTES + 2 * TC_B_BYTES;
constexpr size_t TC_SMEM = 2 * TC_STAGE + 2 * TC_R_BYTES;

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

// CTA (point tile, frequency group), the groups of one tile adjacent in
// blockIdx.x so the tile's samples are read from HBM once.  Eight warps: all
// split samples into A; warp w reads TMEM lanes 32 (w % 4) .. +31 and the
// w / 4 half of the columns in the epilogue.  The samples of a chunk (8 rows
// of 128 points, 1 KB each; P is even, so every row starts 16-byte aligned)
// and its B operands are bulk-copied one chunk ahead.
__global__ void __launch_bounds__(TC_THREADS) k_dft_tc(const float2* __restrict__ S, long P, int nk,
                                                       const float* __restrict__ Bt, int nof, int ngroups,
                                                       double2* __restrict__ fd, int* err) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ uint64_t bar_in[2], bar_mma[2];
  __shared__ uint32_t taddr_s;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int g = blockIdx.x % ngroups;
  const long p0 = (long)(blockIdx.x / ngroups) * TC_M;
  const int np = (int)min((long)TC_M, P - p0);  // points of this tile (even)
  const int nw = min(TC_NW, nof - g * TC_NW);   // frequencies of this group
  const int ncol = ((2 * nw + 15) / 16) * 16;   // MMA N: a multiple of 16
  const int nch = (2 * nk + TC_KC - 1) / TC_KC;
  const long per = (long)TC_BROWS * TC_KC;
  unsigned char* raw = smem + 2 * TC_STAGE;
  if (tid == 0) {
    for (int s = 0; s < 2; ++s) {
      mbar_init(&bar_in[s], 1);
      mbar_init(&bar_mma[s], 1);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&taddr_s)),
                 "r"(TC_NMAX)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = taddr_s;
  const uint32_t idesc = tc_idesc(ncol);
  const unsigned nb = (unsigned)(ncol * TC_KC * 4);
  // chunk c's inputs (its raw samples and B operands) into slot s
  auto issue = [&](int c, int s) {
    const int k0 = c * (TC_KC / 2), nr = min(TC_KC / 2, nk - k0);
    unsigned char* st = smem + s * TC_STAGE;
    const float* src = Bt + ((long)(g * nch + c) * 2) * per;
    mbar_expect_tx(&bar_in[s], 2 * nb + (unsigned)(nr * np * 8));
    fence_proxy_async();
    bulk_g2s(st + 2 * TC_A_BYTES, src, nb, &bar_in[s]);
    bulk_g2s(st + 2 * TC_A_BYTES + TC_B_BYTES, src + per, nb, &bar_in[s]);
    for (int r = 0; r < nr; ++r)
      bulk_g2s(raw + s * TC_R_BYTES + (size_t)r * TC_M * 8, S + (long)(k0 + r) * P + p0, (unsigned)(np * 8),
               &bar_in[s]);
  };
  unsigned par_in = 0, par_mma = 0;
  bool bad = false;
  if (tid == 0) issue(0, 0);
  for (int c = 0; c < nch; ++c) {
    const int s = c & 1;
    unsigned char* st = smem + s * TC_STAGE;
    float* Ah = (float*)st;
    float* Al = (float*)(st + TC_A_BYTES);
    const float* Bh = (const float*)(st + 2 * TC_A_BYTES);
    const float* Bl = (const float*)(st + 2 * TC_A_BYTES + TC_B_BYTES);
    if (c + 1 < nch) {
      // slot s^1 was last read by the MMAs of chunk c-1 (its raw samples by
      // this CTA's split of chunk c-1, finished at that iteration's barrier)
      if (c >= 1) {
        bad |= !mbar_wait(&bar_mma[s ^ 1], (par_mma >> (s ^ 1)) & 1u, STREAM_WAIT_CYCLES);
        par_mma ^= 1u << (s ^ 1);
      }
      if (tid == 0) issue(c + 1, s ^ 1);
    }
    bad |= !mbar_wait(&bar_in[s], (par_in >> s) & 1u, STREAM_WAIT_CYCLES);
    par_in ^= 1u << s;
    // split: thread (row, half) takes samples 4 half .. 4 half + 3 of the chunk
    {
      const int row = tid & (TC_M - 1), half = tid >> 7;
      const int k0 = c * (TC_KC / 2);
      const float2* rw = (const float2*)(raw + s * TC_R_BYTES);
#pragma unroll
      for (int q = 0; q < 2; ++q) {
        const int kq = 4 * half + 2 * q;  // sample pair kq, kq+1 of the chunk
        float2 a = make_float2(0.f, 0.f), b = make_float2(0.f, 0.f);
        if (row < np) {
          if (k0 + kq < nk) a = rw[kq * TC_M + row];
          if (k0 + kq + 1 < nk) b = rw[(kq + 1) * TC_M + row];
        }
        const float4 v = make_float4(a.x, a.y, b.x, b.y);
        const float4 h = make_float4(tf32_hi(v.x), tf32_hi(v.y), tf32_hi(v.z), tf32_hi(v.w));
        *(float4*)(Ah + tc_off(row, 2 * kq)) = h;
        *(float4*)(Al + tc_off(row, 2 * kq)) = make_float4(v.x - h.x, v.y - h.y, v.z - h.z, v.w - h.w);
      }
    }
    fence_proxy_async();  // generic-proxy writes of A before the tensor core reads them
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
      for (int ks = 0; ks < TC_KC / 8; ++ks) {
        const uint64_t ah = tc_desc(Ah + 64 * ks), al = tc_desc(Al + 64 * ks);
        const uint64_t bh = tc_desc(Bh + 64 * ks), bl = tc_desc(Bl + 64 * ks);
        tc_mma(tmem, ah, bh, idesc, (c > 0 || ks > 0) ? 1 : 0);
        tc_mma(tmem, ah, bl, idesc, 1);
        tc_mma(tmem, al, bh, idesc, 1);
      }
      tc_commit(&bar_mma[s]);
    }
  }
  // the commits of the last two chunks (each covers every earlier MMA)
  for (int c = max(0, nch - 2); c < nch; ++c) {
    const int s = c & 1;
    bad |= !mbar_wait(&bar_mma[s], (par_mma >> s) & 1u, STREAM_WAIT_CYCLES);
    par_mma ^= 1u << s;
  }
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (__syncthreads_or(bad)) {
    if (tid == 0) atomicExch(err, 3);
  } else {
    // epilogue: lanes 32 (w % 4) + lane = points, columns of half w / 4
    const int q4 = warp & 3, hw = warp >> 2;
    const int row = 32 * q4 + lane;
    const long pp = p0 + row;
    const int cbeg = hw * (ncol / 2), cend = cbeg + ncol / 2;  // ncol / 2 is a multiple of 8
    for (int c0 = cbeg; c0 < cend; c0 += 16) {
      uint32_t r[16];
      const uint32_t ta = tmem + ((uint32_t)(32 * q4) << 16) + (uint32_t)c0;
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
          : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
            "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
          : "r"(ta)
          : "memory");
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      if (row < np) {
        const int j0 = c0 / 2, jn = min(8, min(nw, cend / 2) - j0);
        double2 f[8];
#pragma unroll
        for (int j = 0; j < 8; ++j)
          if (j < jn) f[j] = fd[(long)(g * TC_NW + j0 + j) * P + pp];
#pragma unroll
        for (int j = 0; j < 8; ++j)
          if (j < jn) {
            f[j].x += (double)__uint_as_float(r[2 * j]);
            f[j].y += (double)__uint_as_float(r[2 * j + 1]);
            fd[(long)(g * TC_NW + j0 + j) * P + pp] = f[j];
          }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TC_NMAX) : "memory");
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

// Poynting flux of one face, code/dataprocess.f90:246-277:
// J = sign * sum Re(a*conj(b) - c*conj(d)) * eps0*Q/(2 dt).
struct FluxFace {
  long pa, pb, pc, pd;  // first sample index of the four components
  long n;               // locations on the face
  int sign, active;
};

__global__ void __launch_bounds__(256) k_flux(const double2* __restrict__ fd, long P, const FluxFace* __restrict__ faces,
                                              int nof, double scale, double* __restrict__ J) {
  __shared__ double red[256];
  const int iw = blockIdx.x, f = blockIdx.y;
  const FluxFace F = faces[f];
  double s = 0.0;
  if (F.active) {
    const double2* row = fd + (long)iw * P;
    for (long L = threadIdx.x; L < F.n; L += blockDim.x) {
      const double2 a = row[F.pa + L], b = row[F.pb + L], c = row[F.pc + L], d = row[F.pd + L];
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
// Fused E+H pass (FP32, IRIS_STENCIL_FUSED).
//
// One pass per time step from (E, H, D) into double buffers (E', H', D'):
// each field value is read once and written once per step (12 complex values
// per cell instead of the split passes' 18).  A CTA is 16 warps; warp w holds
// row y0 + w and lane l column x0 + l of a 32 x 16 tile, and the CTA marches z
// over a chunk of planes.  At plane z every thread computes E'(z) of its cell
// and H'(z-1) of the cell below it, so H' has E'(z-1) and E'(z) at hand: the
// x neighbours come from the next / previous lane by warp shuffle, the y
// neighbours from the next / previous warp through one shared-memory row
// exchange per plane (one barrier).  Tiles overlap by one column and one row:
// lane 31 and the last warp compute the E' that H' needs at +x / +y but write
// nothing, so tiles advance by 31 x 15 and no CTA reads another's output.
// Cells one past nx or ny, and plane nz+1, are the Bloch images of x = 1,
// y = 1, z = 1: their threads compute E' at the image cell and apply the
// phase.  TF/SF and the DFT sample follow as their own kernels on the new
// buffers, as after the split passes.  B is touched only by its owner and
// stays in place; D is double buffered because image and overlap threads
// read the old D of cells another CTA owns.

constexpr int FZ_X = 32, FZ_Y = 16, FZ_OX = FZ_X - 1, FZ_OY = FZ_Y - 1;

struct FusedArgs {
  FieldArgs<float> f;  // the old state: f.e, f.h, f.pml_d (D old), f.pml_b (B, in place)
  float2* e_new;
  float2* h_new;
  float2* d_new[2];
  int zchunk;  // planes per CTA
};

__device__ __forceinline__ cx<float> shfl_cx(cx<float> v, int d, bool up) {
  cx<float> r;
  r.re = up ? __shfl_up_sync(0xffffffffu, v.re, d) : __shfl_down_sync(0xffffffffu, v.re, d);
  r.im = up ? __shfl_up_sync(0xffffffffu, v.im, d) : __shfl_down_sync(0xffffffffu, v.im, d);
  return r;
}

template <bool CEPS> __global__ void __launch_bounds__(FZ_X* FZ_Y, 2) k_fused(FusedArgs A) {
  const FieldArgs<float>& a = A.f;
  const Geo& g = a.g;
  // per row and plane parity: H(z) components 1, 3 and E'(z-1) components 1, 3
  __shared__ float2 xr[2][FZ_Y][4][FZ_X];
  const int lane = threadIdx.x, w = threadIdx.y;
  const int x = 1 + blockIdx.x * FZ_OX + lane, y = 1 + blockIdx.y * FZ_OY + w;
  const int z0 = 1 + blockIdx.z * A.zchunk, z1 = min(z0 + A.zchunk - 1, g.nz);
  const bool act = x <= g.nx + 1 && y <= g.ny + 1;
  const bool ximg = x == g.nx + 1, yimg = y == g.ny + 1;
  const int cxx = ximg ? 1 : x, cyy = yimg ? 1 : y;  // the cell whose E' this thread computes
  const bool own = lane < FZ_OX && w < FZ_OY && x <= g.nx && y <= g.ny;
  cx<float> ph = {1.f, 0.f};
  if (ximg) ph = cmul(ph, a.pxp);
  if (yimg) ph = cmul(ph, a.pyp);
  const float2* E = a.e;
  const float2* H = a.h;
  auto ldc = [&](const float2* f, int k, int xx, int yy, int zz) {
    return ld<float>(f + k * g.comp + g.at(xx, yy, zz));
  };
  const cx<float> zero = {0.f, 0.f};
  // Carried from plane z-1 in this thread's own slots of the exchange rows
  // (written there for the neighbours anyway): components 1, 3 of H(z-1) in
  // rows of parity (z-1)&1 and of E'(z-1) in rows of parity z&1 (stored at
  // the end of the previous plane); component 2 of both in registers.
  cx<float> ep1 = zero, hp1 = act ? ldc(H, 1, cxx, cyy, z0 - 1) : zero;
  {
    const cx<float> h0 = act ? ldc(H, 0, cxx, cyy, z0 - 1) : zero, h2 = act ? ldc(H, 2, cxx, cyy, z0 - 1) : zero;
    xr[(z0 - 1) & 1][w][0][lane] = make_float2(h0.re, h0.im);
    xr[(z0 - 1) & 1][w][1][lane] = make_float2(h2.re, h2.im);
    xr[z0 & 1][w][2][lane] = make_float2(0.f, 0.f);
    xr[z0 & 1][w][3][lane] = make_float2(0.f, 0.f);
  }
  cx<float> en[3], hn_[3];  // E and H of the next plane, loaded one plane ahead
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    en[k] = act ? ldc(E, k, cxx, cyy, z0) : zero;
    hn_[k] = act ? ldc(H, k, cxx, cyy, z0) : zero;
  }
  for (int z = z0; z <= z1 + 1; ++z) {
    const int buf = z & 1;
    const bool zimg = z == g.nz + 1;
    const int cz = zimg ? 1 : z;
    cx<float> e[3], h[3], hzm0, hzm1, ep[3], hp[3];
    {
      const float2 a0 = xr[buf ^ 1][w][0][lane], a2 = xr[buf ^ 1][w][1][lane];
      const float2 b0 = xr[buf][w][2][lane], b2 = xr[buf][w][3][lane];
      hp[0] = {a0.x, a0.y};
      hp[1] = hp1;
      hp[2] = {a2.x, a2.y};
      ep[0] = {b0.x, b0.y};
      ep[1] = ep1;
      ep[2] = {b2.x, b2.y};
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      e[k] = en[k];
      h[k] = hn_[k];
    }
    if (act && z + 1 <= z1 + 1) {
      const int zn = z + 1 == g.nz + 1 ? 1 : z + 1;
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        en[k] = ldc(E, k, cxx, cyy, zn);
        hn_[k] = ldc(H, k, cxx, cyy, zn);
      }
    }
    if (zimg && act) {
      hzm0 = ldc(H, 0, cxx, cyy, 0);
      hzm1 = ldc(H, 1, cxx, cyy, 0);
    } else {
      hzm0 = hp[0];
      hzm1 = hp[1];
    }
    xr[buf][w][0][lane] = make_float2(h[0].re, h[0].im);
    xr[buf][w][1][lane] = make_float2(h[2].re, h[2].im);
    cx<float> hx1 = shfl_cx(h[1], 1, true), hx2 = shfl_cx(h[2], 1, true);
    const cx<float> ex1 = shfl_cx(ep[1], 1, false), ex2 = shfl_cx(ep[2], 1, false);
    __syncthreads();
    cx<float> enew[3];
    if (act) {
      if (lane == 0 || ximg) {
        hx1 = ldc(H, 1, cxx - 1, cyy, cz);
        hx2 = ldc(H, 2, cxx - 1, cyy, cz);
      }
      cx<float> hy0, hy2;
      if (w == 0 || yimg) {
        hy0 = ldc(H, 0, cxx, cyy - 1, cz);
        hy2 = ldc(H, 2, cxx, cyy - 1, cz);
      } else {
        const float2 u = xr[buf][w - 1][0][lane], v = xr[buf][w - 1][1][lane];
        hy0 = {u.x, u.y};
        hy2 = {v.x, v.y};
      }
      // the curl of e_update, then its material / UPML part
      cx<float> c[3];
      c[0] = cadd(csub(csub(h[2], hy2), h[1]), hzm1);
      c[1] = cadd(csub(csub(h[0], hzm0), h[2]), hx2);
      c[2] = cadd(csub(csub(h[1], hx1), h[0]), hy0);
#pragma unroll
      for (int k = 0; k < 3; ++k) enew[k] = e[k];
      e_apply<float, CEPS>(a, (own && z <= z1) ? A.d_new : nullptr, cxx, cyy, cz, c, enew);
      if (ximg || yimg) {
#pragma unroll
        for (int k = 0; k < 3; ++k) enew[k] = cmul(ph, enew[k]);
      }
      if (zimg) {
#pragma unroll
        for (int k = 0; k < 3; ++k) enew[k] = cmul(a.pzp, enew[k]);
      }
      if (own && z > z0) {
        // H'(z-1) of (x, y): h_update from E'(z-1), its +x and +y neighbours and E'(z)
        cx<float> xp[3], yp[3], zp[3], hn[3];
        xp[1] = ex1;
        xp[2] = ex2;
        const float2 u = xr[buf][w + 1][2][lane], v = xr[buf][w + 1][3][lane];
        yp[0] = {u.x, u.y};
        yp[2] = {v.x, v.y};
        zp[0] = enew[0];
        zp[1] = enew[1];
#pragma unroll
        for (int k = 0; k < 3; ++k) hn[k] = hp[k];
        h_update<float>(a, x, y, z - 1, ep, xp, yp, zp, hn);
        const long i = g.at(x, y, z - 1);
#pragma unroll
        for (int k = 0; k < 3; ++k) st<float>(A.h_new + k * g.comp + i, hn[k]);
        if (x == g.nx) {
          const long q = g.at(0, y, z - 1);
#pragma unroll
          for (int k = 0; k < 3; ++k) {
            st<float>(A.e_new + k * g.comp + q, cmul(a.pxm, ep[k]));
            st<float>(A.h_new + k * g.comp + q, cmul(a.pxm, hn[k]));
          }
        }
        if (y == g.ny) {
          const long q = g.at(x, 0, z - 1);
#pragma unroll
          for (int k = 0; k < 3; ++k) {
            st<float>(A.e_new + k * g.comp + q, cmul(a.pym, ep[k]));
            st<float>(A.h_new + k * g.comp + q, cmul(a.pym, hn[k]));
          }
        }
        if (z - 1 == g.nz) {
          const long q = g.at(x, y, 0);
#pragma unroll
          for (int k = 0; k < 3; ++k) {
            st<float>(A.e_new + k * g.comp + q, cmul(a.pzm, ep[k]));
            st<float>(A.h_new + k * g.comp + q, cmul(a.pzm, hn[k]));
          }
        }
      }
      if (own && z <= z1) {
        const long i = g.at(x, y, z);
#pragma unroll
        for (int k = 0; k < 3; ++k) st<float>(A.e_new + k * g.comp + i, enew[k]);
        if (x == 1) {
          const long q = g.at(g.nx + 1, y, z);
#pragma unroll
          for (int k = 0; k < 3; ++k) st<float>(A.e_new + k * g.comp + q, cmul(a.pxp, enew[k]));
        }
        if (y == 1) {
          const long q = g.at(x, g.ny + 1, z);
#pragma unroll
          for (int k = 0; k < 3; ++k) st<float>(A.e_new + k * g.comp + q, cmul(a.pyp, enew[k]));
        }
        if (z == 1) {
          const long q = g.at(x, y, g.nz + 1);
#pragma unroll
          for (int k = 0; k < 3; ++k) st<float>(A.e_new + k * g.comp + q, cmul(a.pzp, enew[k]));
        }
      }
    } else {
#pragma unroll
      for (int k = 0; k < 3; ++k) enew[k] = zero;
    }
    // carry E'(z) to the next plane: components 1, 3 into the rows of the
    // other parity (last read during plane z-1, before this plane's barrier)
    xr[buf ^ 1][w][2][lane] = make_float2(enew[0].re, enew[0].im);
    xr[buf ^ 1][w][3][lane] = make_float2(enew[2].re, enew[2].im);
    ep1 = enew[1];
    hp1 = h[1];
  }
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

#define CK(call)                                                                                      \
  do {                                                                                                \
    cudaError_t err_ = (call);                                                                        \
    if (err_ != cudaSuccess)                                                                          \
      return fail(err_ == cudaErrorMemoryAllocation ? IRIS_ENOMEM : IRIS_ECUDA,                      \
                  std::string(#call) + ": " + cudaGetErrorString(err_));                              \
  } while (0)


namespace {

struct FaceMap {
  bool active = false;  // this face pair is accumulated by scattering_fourier
  int nu = 0, nv = 0;
  long nloc = 0;         // locations per face
  long base[2][6] = {};  // first sample index per [side][component]
};

}  // namespace

struct iris_engine {
  iris_params p{};
  std::vector<double> fw;
  int prec = IRIS_FP64;
  size_t esz = 16;  // bytes per stored complex value
  int device = 0;
  cudaStream_t st = nullptr;
  Geo g{};
  dim3 blk, grd;
  void* e = nullptr;
  void* h = nullptr;
  void* pml_d[2] = {nullptr, nullptr};
  void* pml_b[2] = {nullptr, nullptr};
  long pcomp[2] = {0, 0};
  int nbot = 0, ntop = 0;
  void* coef = nullptr;
  std::vector<double> coef_h;
  void* eps = nullptr;
  bool eps_complex = false;
  double ph[6][2] = {};  // exp(+i akx), exp(+i aky), exp(+i akz), exp(-i akx), ...
  SrcArgs src{};
  dim3 tf_blk, tf_grd;
  // DFT
  int nboxes = 1;
  FaceMap fm[2][3];
  long P = 0;
  int K = 0, nslot = 0;
  std::vector<Seg> segs;
  long max_seg = 0;
  Seg* d_segs = nullptr;
  void* S = nullptr;
  int* d_tk = nullptr;
  double* d_fw = nullptr;
  double2* fd = nullptr;
  float2* d_wt = nullptr;
  double2* d_wt64 = nullptr;  // FP64 mode twiddles of one block
  bool dft_tc = false;     // FP32 block accumulation on the tensor cores
  float* d_wtc = nullptr;  // its B operands (k_twiddle_tc)
  FluxFace* d_faces = nullptr;
  double* d_J = nullptr;
  double* h_J = nullptr;
  // batch member: no DFT buffers of its own; z-plane DFT only on request
  bool member = false;
  bool dft_z_only = false;
  std::vector<FluxFace> host_faces;
  // fused E+H stepping (FP32): second field buffers and D, per-step TF/SF table
  bool fused = false;
  void* e2 = nullptr;
  void* h2 = nullptr;
  void* pml_d2[2] = {nullptr, nullptr};
  int zchunk = 0;
  dim3 fblk, fgrd;
  // CUDA graph of one DFT block of steps (iris_params.graph): d_it holds the
  // step base the captured kernels add to their offsets, dev_it its value
  cudaGraphExec_t gexec = nullptr;
  int* d_it = nullptr;
  int dev_it = -1;
  // streamed split passes (FP32, real material); d_err: a kernel's give-up record
  bool stream = false;
  dim3 sgrd;
  int* d_err = nullptr;
  // timing: CUDA events on the engine stream, per kernel class
  bool timing = false;
  cudaEvent_t t0 = nullptr, t1 = nullptr;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> ev[IRIS_NKC];
  size_t ev_used[IRIS_NKC] = {};
};

namespace {

// Brackets one kernel launch with a pair of events when timing is on.
struct KTimer {
  iris_engine* E;
  int k;
  cudaEvent_t b = nullptr, e = nullptr;
  KTimer(iris_engine* eng, int kind) : E(eng), k(kind) {
    if (!E->timing) return;
    auto& v = E->ev[k];
    if (E->ev_used[k] == v.size()) {
      cudaEvent_t x, y;
      cudaEventCreate(&x);
      cudaEventCreate(&y);
      v.push_back({x, y});
    }
    b = v[E->ev_used[k]].first;
    e = v[E->ev_used[k]].second;
    ++E->ev_used[k];
    cudaEventRecord(b, E->st);
  }
  ~KTimer() {
    if (b) cudaEventRecord(e, E->st);
  }
};

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
  if (p.stencil < IRIS_STENCIL_DEFAULT || p.stencil > IRIS_STENCIL_STREAM) return bad("unknown stencil variant");
  if (p.stencil == IRIS_STENCIL_FUSED && p.precision != IRIS_FP32) return bad("the fused stencil is FP32 only");
  if (p.stencil == IRIS_STENCIL_STREAM && p.precision != IRIS_FP32) return bad("the streamed stencil is FP32 only");
  if (p.dft_faces != IRIS_DFT_ALL && p.dft_faces != IRIS_DFT_Z) return bad("dft_faces must be IRIS_DFT_ALL or IRIS_DFT_Z");
  if (p.dft_kernel < IRIS_DFT_KERNEL_AUTO || p.dft_kernel > IRIS_DFT_KERNEL_TENSOR) return bad("unknown dft_kernel");
  return IRIS_OK;
}

template <typename T> FieldArgs<T> field_args(const iris_engine* E) {
  using V = typename V2<T>::t;
  const iris_params& p = E->p;
  FieldArgs<T> a{};
  a.e = (V*)E->e;
  a.h = (V*)E->h;
  a.g = E->g;
  for (int s = 0; s < 2; ++s) {
    a.pml_d[s] = (V*)E->pml_d[s];
    a.pml_b[s] = (V*)E->pml_b[s];
    a.pcomp[s] = E->pcomp[s];
  }
  a.coef = (const T*)E->coef;
  a.pmlzi = p.pmlzi;
  a.pmlzf = p.pmlzf;
  a.hi = p.hi;
  a.hf = p.hf;
  a.eps_c = E->eps_complex ? (const V*)E->eps : nullptr;
  a.eps_r = E->eps_complex ? nullptr : (const T*)E->eps;
  a.m1 = (T)(1.0 / p.eps1);
  a.m3 = (T)(1.0 / p.eps3);
  a.eps0sq = (T)(p.eps0 * p.eps0);
  const double dtc = p.dt * p.c0 / p.Q;
  a.dtcq2 = (T)(dtc * dtc);
  cx<T>* ph[6] = {&a.pxp, &a.pyp, &a.pzp, &a.pxm, &a.pym, &a.pzm};
  for (int k = 0; k < 6; ++k) *ph[k] = cx<T>{(T)E->ph[k][0], (T)E->ph[k][1]};
  return a;
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

void dft_flush(iris_engine* E) {
  if (E->nslot == 0) return;
  KTimer tm(E, IRIS_KC_DFT);
  const int nk = E->nslot;
  if (E->prec == IRIS_FP64) {
    const int nwc = (E->p.nof + DFT64_WC - 1) / DFT64_WC;
    const long nblk = (E->P + 127) / 128;
    k_twiddle64<<<(nk * E->p.nof + 255) / 256, 256, 0, E->st>>>(E->d_tk, nk, E->d_fw, E->p.nof, E->d_wt64);
    k_dft_fp64<<<(unsigned)(nblk * nwc), 128, (size_t)nk * DFT64_WC * sizeof(double2), E->st>>>(
        (const double2*)E->S, E->P, nk, E->d_wt64, E->p.nof, nwc, E->p.dt, E->fd);
  } else if (E->dft_tc) {
    const int ng = (E->p.nof + TC_NW - 1) / TC_NW, nch = (2 * nk + TC_KC - 1) / TC_KC;
    const long nt = (long)ng * nch * TC_BROWS * TC_KC;
    k_twiddle_tc<<<(unsigned)((nt + 255) / 256), 256, 0, E->st>>>(E->d_tk, 0, 0, nk, E->d_fw, E->p.nof, E->p.dt, ng,
                                                                   nch, E->d_wtc);
    const long ntiles = (E->P + TC_M - 1) / TC_M;
    k_dft_tc<<<(unsigned)(ntiles * ng), TC_THREADS, TC_SMEM, E->st>>>((const float2*)E->S, E->P, nk, E->d_wtc,
                                                                       E->p.nof, ng, E->fd, E->d_err);
  } else {
    const int nt = nk * E->p.nof;
    k_twiddle<<<(nt + 255) / 256, 256, 0, E->st>>>(E->d_tk, 0, 0, nk, E->d_fw, E->p.nof, E->p.dt, E->d_wt);
    const int nwc = (E->p.nof + DFT_TW - 1) / DFT_TW;
    const long nblk = (E->P + DFT_TP - 1) / DFT_TP;
    k_dft_fp32<<<(unsigned)(nblk * nwc), DFT_THREADS, 0, E->st>>>((const float2*)E->S, E->P, nk, E->d_wt, E->p.nof, nwc,
                                                        E->fd);
  }
  E->nslot = 0;
}

template <typename T> void dft_sample(iris_engine* E, int t, const int* tp = nullptr) {
  if (E->P == 0) return;
  using V = typename V2<T>::t;
  {
  KTimer tm(E, IRIS_KC_GATHER);
  V* slot = (V*)E->S + (long)E->nslot * E->P;
  dim3 grid((unsigned)((E->max_seg + 255) / 256), (unsigned)E->segs.size());
  k_dft_gather<T><<<grid, 256, 0, E->st>>>((const V*)E->e, (const V*)E->h, E->g.comp, E->d_segs, slot, E->d_tk,
                                          E->nslot, t, tp);
  }
  if (++E->nslot == E->K) dft_flush(E);
}

FusedArgs fused_args(const iris_engine* E) {
  FusedArgs a{};
  a.f = field_args<float>(E);
  a.e_new = (float2*)E->e2;
  a.h_new = (float2*)E->h2;
  for (int s = 0; s < 2; ++s) a.d_new[s] = (float2*)E->pml_d2[s];
  a.zchunk = E->zchunk;
  return a;
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
template <typename F> int graph_block(iris_engine* E, int it, F record) {
  if (!E->d_it) {
    CK(cudaMalloc(&E->d_it, sizeof(int)));
    E->dev_it = -1;
  }
  if (E->dev_it != it) k_set_int<<<1, 1, 0, E->st>>>(E->d_it, it);
  if (!E->gexec) {
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

// One fused step into the second buffers, swap, then TF/SF and the DFT
// sample on the new state, in the operator order of the split passes; step
// it, or *itp + it when itp is given.
void fused_one(iris_engine* E, int it, const int* itp, bool sampled) {
  {
    KTimer tm(E, IRIS_KC_FUSED);
    const FusedArgs a = fused_args(E);
    if (E->eps_complex) k_fused<true><<<E->fgrd, E->fblk, 0, E->st>>>(a);
    else k_fused<false><<<E->fgrd, E->fblk, 0, E->st>>>(a);
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

int alloc_dft(iris_engine* E, const FluxFace* faces, int nfaces);

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
  E->P = P;
  E->host_faces = faces;
  if (E->member) return IRIS_OK;  // a batch member: the batch owns the DFT buffers
  return alloc_dft(E, faces.data(), 12);
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
  // at most 256 slots (the FP64 block kernel stages K x 8 twiddles in 32 KB of
  // shared memory); FP32 defaults to 256 so the FP64 epilogue is amortised
  int K = std::min(256, p.dft_block > 0 ? p.dft_block : (E->prec == IRIS_FP64 ? 32 : 256));
  const size_t slot_bytes = std::max<size_t>(1, (size_t)P * E->esz);
  const size_t budget = (freeb - fd_bytes) / 4;
  while (K > 1 && (size_t)K * slot_bytes > budget) K /= 2;
  E->K = std::max(1, K);
  E->nslot = 0;
  CK(cudaMalloc(&E->fd, std::max<size_t>(fd_bytes, 16)));
  CK(cudaMemsetAsync(E->fd, 0, std::max<size_t>(fd_bytes, 16), E->st));
  CK(cudaMalloc(&E->S, (size_t)E->K * slot_bytes));
  CK(cudaMalloc(&E->d_tk, sizeof(int) * E->K));
  CK(cudaMalloc(&E->d_fw, sizeof(double) * p.nof));
  CK(cudaMemcpy(E->d_fw, E->fw.data(), sizeof(double) * p.nof, cudaMemcpyHostToDevice));
  if (E->prec == IRIS_FP32) CK(cudaMalloc(&E->d_wt, sizeof(float2) * (size_t)E->K * p.nof));
  if (E->prec == IRIS_FP64) CK(cudaMalloc(&E->d_wt64, sizeof(double2) * (size_t)E->K * p.nof));
  E->dft_tc = E->prec == IRIS_FP32 && p.dft_kernel != IRIS_DFT_KERNEL_CUDA;
  if (E->dft_tc) {
    const int ng = (p.nof + TC_NW - 1) / TC_NW, nch = (2 * E->K + TC_KC - 1) / TC_KC;
    CK(cudaMalloc(&E->d_wtc, sizeof(float) * (size_t)ng * nch * 2 * TC_BROWS * TC_KC));
    CK(cudaFuncSetAttribute(k_dft_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TC_SMEM));
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
                  E->pml_d2[1], E->d_err, E->d_it, E->d_wtc, E->d_wt64};
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
  if (E->st) cudaStreamDestroy(E->st);
}

}  // namespace

long iris::engine_npts(const iris_engine* E, int box, int j) {
  if (box < 0 || box >= E->nboxes || j < 1 || j > 3) return 0;
  const FaceMap& F = E->fm[box][j - 1];
  return F.active ? 12 * F.nloc : 0;
}

extern "C" {

static int create_engine(const iris_params* pin, const double* fw, bool member, bool z_only, iris_engine** out,
                         bool packed = false);

int iris_create(const iris_params* pin, const double* fw, iris_engine** out) {
  return create_engine(pin, fw, false, false, out);
}

}  // extern "C"

// packed: rows of nx+2 cells back to back (no 128-byte alignment of x = 1),
// for cells whose rows are short; component arrays stay 128-byte aligned.
static int create_engine(const iris_params* pin, const double* fw, bool member, bool z_only, iris_engine** out,
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
  // fused E+H pass: FP32 only
  // fused on request only: it moves fewer bytes but issues ~1.6x the
  // instructions of the split passes and measures slower on GB300 for now
  // FP32 steps with the fused pass unless the split or streamed passes are asked for
  E->fused = E->prec == IRIS_FP32 && (p.stencil == IRIS_STENCIL_FUSED || p.stencil == IRIS_STENCIL_DEFAULT);
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
    // z chunks: about eight waves of two CTAs per SM, at least 16 planes each
    const long tiles = (long)((p.nx + FZ_OX - 1) / FZ_OX) * ((p.ny + FZ_OY - 1) / FZ_OY);
    long nch = std::max(1L, (8L * 152 * 2 + tiles - 1) / tiles);
    nch = std::min<long>(nch, std::max(1, p.nz / 16));
    E->zchunk = (int)((p.nz + nch - 1) / nch);
    E->fblk = dim3(FZ_X, FZ_Y, 1);
    E->fgrd = dim3((p.nx + FZ_OX - 1) / FZ_OX, (p.ny + FZ_OY - 1) / FZ_OY, (p.nz + E->zchunk - 1) / E->zchunk);
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

// Status of the engine's bounded device waits: IRIS_ETIMEOUT once a kernel
// gave up on one (the stream is synchronised first).
static int stream_status(iris_engine* E) {
  if (!E->d_err) return IRIS_OK;
  int h = 0;
  CK(cudaMemcpyAsync(&h, E->d_err, sizeof(int), cudaMemcpyDeviceToHost, E->st));
  CK(cudaStreamSynchronize(E->st));
  if (h) return fail(IRIS_ETIMEOUT, h == 3 ? std::string("the tensor-core DFT block gave up waiting")
                                            : std::string("a streamed ") + (h == 1 ? "E" : "H") +
                                                  " pass gave up waiting for its staged plane");
  return IRIS_OK;
}

extern "C" {

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

int iris_step(iris_engine* E, int it0, int nsteps) {
  clear_error();
  if (!E || nsteps < 0) return fail(IRIS_EINVAL, "bad argument");
  CK(cudaSetDevice(E->device));
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
  clear_error();
  if (!E || !J || box < 0 || box > 1) return fail(IRIS_EINVAL, "bad argument");
  CK(cudaSetDevice(E->device));
  const iris_params& p = E->p;
  if (box >= E->nboxes) box = 0;  // a single box: the second one is the same box
  dft_flush(E);
  const double scale = p.eps0 * p.Q / (2.0 * p.dt);
  KTimer tm(E, IRIS_KC_FLUX);
  k_flux<<<dim3(p.nof, 6), 256, 0, E->st>>>(E->fd, E->P, E->d_faces + 6 * box, p.nof, scale, E->d_J);
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
  if (!finite) return fail(IRIS_ENAN, "non-finite flux");
  return IRIS_OK;
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
  const int nof = E->p.nof;
  std::vector<double2> row((size_t)E->P);
  for (int iw = 0; iw < nof; ++iw) {
    CK(cudaMemcpyAsync(row.data(), E->fd + (size_t)iw * E->P, sizeof(double2) * E->P, cudaMemcpyDeviceToHost, E->st));
    CK(cudaStreamSynchronize(E->st));
    for (int side = 0; side < 2; ++side)
      for (int ip = 0; ip < 6; ++ip)
        for (long L = 0; L < F.nloc; ++L) {
          const long q = side * 6 * F.nloc + ip + 6 * L;
          const double2 v = row[F.base[side][ip] + L];
          re[(size_t)iw * n + q] = v.x;
          im[(size_t)iw * n + q] = v.y;
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
    default: return fail(IRIS_EINVAL, "unknown operator");
  }
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(E->st));
  return IRIS_OK;
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
  if (!samples || !fw || !fdata) return fail(IRIS_EINVAL, "iris_dft_block_noalloc: null device pointer");
  if (nk < 1 || npts < 1 || nof < 1) return fail(IRIS_EINVAL, "iris_dft_block_noalloc: nk, npts and nof must be >= 1");
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
  k_dft_fp32<<<(unsigned)(nblk * nwc), DFT_THREADS, 0, st>>>((const float2*)samples, npts, nk, (const float2*)wt, nof,
                                                           nwc, (double2*)fdata);
  CK(cudaGetLastError());
  return IRIS_OK;
}

// ---------------------------------------------------------------------------
// Batched form: many independent Bloch cells (or k-points) stepped together.
//
// Each cell is a member engine (its own fields, UPML, material, source and
// DFT point layout, but no DFT buffers).  One launch per operator covers
// every cell: a persistent kernel walks a work list of (cell, tile) items in
// cell, z, y, x order, so the CTAs running together touch neighbouring tiles
// of one cell and the neighbour loads hit L2.  The DFT samples of all cells go
// to one shared ring and one accumulator array (all cells share dt and the
// frequency list) and are accumulated by the single-engine block kernel.  The
// tile shape is picked by iris_batch_tune, which times the candidates on the
// batch itself.

namespace iris {
namespace {

struct BItem {
  int cell, x0, y0, z0;  // tile origin (1-based)
};
struct TItem {
  int cell, ix0, iy0, pad;
};
struct BSeg {
  Seg s;
  int cell, pad;
};

// Work-list shapes the autotuner chooses from: x * y * z blocks of cells,
// and (FLAT) 256 consecutive cells of one plane in row-major order, which
// keeps every lane busy whatever the cell's nx.
// keeps every lane busy whatever the cell's nx (FLAT: register-capped for
// five resident blocks per SM; FLAT + 1: uncapped).
constexpr int NTILES = 7, FLAT = 5;
constexpr int TILES[NTILES][3] = {{32, 8, 1}, {32, 4, 2}, {64, 4, 1}, {16, 16, 1}, {32, 2, 4}, {256, 1, 1}, {256, 1, 1}};

// Copies the cell's arguments into shared memory when the item's cell changes.
template <typename A>
__device__ __forceinline__ void cell_args(const A* args, int cell, A& sa, int& scell, int tid) {
  if (cell != scell) {
    __syncthreads();
    if (tid == 0) {
      sa = args[cell];
      scell = cell;
    }
    __syncthreads();
  }
}

template <typename T, int TX, int TY, int TZ>
__global__ void __launch_bounds__(TX* TY* TZ) k_batch_e(const FieldArgs<T>* __restrict__ args,
                                                        const BItem* __restrict__ items, long nitems) {
  __shared__ FieldArgs<T> sa;
  __shared__ int scell;
  const int tid = (threadIdx.z * TY + threadIdx.y) * TX + threadIdx.x;
  if (tid == 0) scell = -1;
  __syncthreads();
  for (long k = blockIdx.x; k < nitems; k += gridDim.x) {
    const BItem b = items[k];
    cell_args(args, b.cell, sa, scell, tid);
    const int x = b.x0 + threadIdx.x, y = b.y0 + threadIdx.y, z = b.z0 + threadIdx.z;
    if (x <= sa.g.nx && y <= sa.g.ny && z <= sa.g.nz) {
      if (sa.eps_c) e_split_cell<T, true>(sa, x, y, z);
      else e_split_cell<T, false>(sa, x, y, z);
    }
  }
}

template <typename T, int TX, int TY, int TZ>
__global__ void __launch_bounds__(TX* TY* TZ) k_batch_h(const FieldArgs<T>* __restrict__ args,
                                                        const BItem* __restrict__ items, long nitems) {
  __shared__ FieldArgs<T> sa;
  __shared__ int scell;
  const int tid = (threadIdx.z * TY + threadIdx.y) * TX + threadIdx.x;
  if (tid == 0) scell = -1;
  __syncthreads();
  for (long k = blockIdx.x; k < nitems; k += gridDim.x) {
    const BItem b = items[k];
    cell_args(args, b.cell, sa, scell, tid);
    const int x = b.x0 + threadIdx.x, y = b.y0 + threadIdx.y, z = b.z0 + threadIdx.z;
    if (x <= sa.g.nx && y <= sa.g.ny && z <= sa.g.nz) h_split_cell<T>(sa, x, y, z);
  }
}

// FLAT items: x0 = first row-major offset in the plane, z0 = the plane.
// MINB: resident blocks per SM asked of the register allocator (0: none).
// CEPS: some cell has a complex material (else every eps_c is null).
// UPML = false: every item's plane lies outside its cell's UPML slabs.
template <typename T, bool EPASS, int MINB, bool CEPS, bool UPML>
__global__ void __launch_bounds__(256, MINB) k_batch_flat(const FieldArgs<T>* __restrict__ args,
                                                    const BItem* __restrict__ items, long nitems) {
  __shared__ FieldArgs<T> sa;
  __shared__ int scell;
  const int tid = threadIdx.x;
  if (tid == 0) scell = -1;
  __syncthreads();
  // the next item's descriptor is loaded while this one is processed
  BItem nb = blockIdx.x < nitems ? items[blockIdx.x] : BItem{};
  for (long k = blockIdx.x; k < nitems; k += gridDim.x) {
    const BItem b = nb;
    if (k + gridDim.x < nitems) nb = items[k + gridDim.x];
    cell_args(args, b.cell, sa, scell, tid);
    const int nx = sa.g.nx;
    const int L = b.x0 + tid;
    if (L < nx * sa.g.ny) {
      const int y = L / nx, x = L - y * nx;
      if (EPASS) {
        if (CEPS && sa.eps_c) e_split_cell<T, true, UPML>(sa, x + 1, y + 1, b.z0);
        else e_split_cell<T, false, UPML>(sa, x + 1, y + 1, b.z0);
      } else {
        h_split_cell<T, UPML>(sa, x + 1, y + 1, b.z0);
      }
    }
  }
}

template <typename T>
__global__ void __launch_bounds__(64) k_batch_tfsf(const FieldArgs<T>* __restrict__ args,
                                                   const SrcArgs* __restrict__ srcs, const TItem* __restrict__ items,
                                                   long nitems, int it, const int* itp) {
  if (itp) it += *itp;
  for (long k = blockIdx.x; k < nitems; k += gridDim.x) {
    const TItem b = items[k];
    const FieldArgs<T>& a = args[b.cell];
    const SrcArgs& s = srcs[b.cell];
    const int ix = b.ix0 + threadIdx.x;
    if (s.variant == 0 || ix > s.nx + 1) continue;
    tfsf_column<T>(a.e, a.h, a.g, s, it, ix, b.iy0, min(b.iy0 + TFSF_YCH - 1, s.ny + 1));
  }
}

template <typename T>
__global__ void __launch_bounds__(256) k_batch_gather(const FieldArgs<T>* __restrict__ args,
                                                      const BSeg* __restrict__ segs,
                                                      typename V2<T>::t* __restrict__ slot, int* tk, int islot,
                                                      int t, const int* tp) {
  if (blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0) tk[islot] = tp ? *tp + t : t;
  const BSeg b = segs[blockIdx.y];
  const long L = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (L >= (long)b.s.nu * b.s.nv) return;
  const FieldArgs<T>& a = args[b.cell];
  const int u = (int)(L % b.s.nu), v = (int)(L / b.s.nu);
  const typename V2<T>::t* src = b.s.field < 3 ? a.e + b.s.field * a.g.comp : a.h + (b.s.field - 3) * a.g.comp;
  slot[b.s.p0 + L] = src[b.s.src + (long)u * b.s.su + (long)v * b.s.sv];
}

}  // namespace
}  // namespace iris

struct iris_batch {
  int n = 0;
  int prec = IRIS_FP64;
  int device = 0;
  iris_engine* master = nullptr;  // stream, timing and the shared DFT buffers
  std::vector<iris_engine*> cells;
  std::vector<long> pbase;
  void* d_args = nullptr;  // FieldArgs<T>[n]
  SrcArgs* d_src = nullptr;
  BItem* d_items = nullptr;
  long nitems = 0;
  long nitems_in = 0;  // flat work lists: items outside the UPML slabs come first
  int tile = 0;  // index into TILES
  int grid_e = 0, grid_h = 0;
  TItem* d_titems = nullptr;
  long ntitems = 0;
  BSeg* d_bsegs = nullptr;
  int nbsegs = 0;
  long max_seg = 0;
  long steps_taken = 0;
};

namespace {

int batch_upload_args(iris_batch* B) {
  const size_t sz = B->prec == IRIS_FP64 ? sizeof(FieldArgs<double>) : sizeof(FieldArgs<float>);
  std::vector<unsigned char> h(sz * B->n);
  for (int c = 0; c < B->n; ++c) {
    if (B->prec == IRIS_FP64) {
      FieldArgs<double> a = field_args<double>(B->cells[c]);
      std::memcpy(h.data() + sz * c, &a, sz);
    } else {
      FieldArgs<float> a = field_args<float>(B->cells[c]);
      std::memcpy(h.data() + sz * c, &a, sz);
    }
  }
  if (!B->d_args) CK(cudaMalloc(&B->d_args, h.size()));
  CK(cudaMemcpy(B->d_args, h.data(), h.size(), cudaMemcpyHostToDevice));
  return IRIS_OK;
}

int batch_build_items(iris_batch* B, int tile) {
  const int TX = TILES[tile][0], TY = TILES[tile][1], TZ = TILES[tile][2];
  std::vector<BItem> items;
  for (int c = 0; c < B->n; ++c) {
    const iris_params& p = B->cells[c]->p;
    if (tile >= FLAT) {
      const int nxy = p.nx * p.ny;
      for (int z = 1; z <= p.nz; ++z)
        if (z > p.pmlzi && z < p.pmlzf)
          for (int l = 0; l < nxy; l += TX) items.push_back(BItem{c, l, 0, z});
      continue;
    }
    for (int z = 1; z <= p.nz; z += TZ)
      for (int y = 1; y <= p.ny; y += TY)
        for (int x = 1; x <= p.nx; x += TX) items.push_back(BItem{c, x, y, z});
  }
  B->nitems_in = tile >= FLAT ? (long)items.size() : 0;
  if (tile >= FLAT)
    for (int c = 0; c < B->n; ++c) {
      const iris_params& p = B->cells[c]->p;
      const int nxy = p.nx * p.ny;
      for (int z = 1; z <= p.nz; ++z)
        if (z <= p.pmlzi || z >= p.pmlzf)
          for (int l = 0; l < nxy; l += TX) items.push_back(BItem{c, l, 0, z});
    }
  graph_reset(B->master);  // captured launches hold the old work list
  if (B->d_items) cudaFree(B->d_items);
  B->d_items = nullptr;
  CK(cudaMalloc(&B->d_items, sizeof(BItem) * items.size()));
  CK(cudaMemcpy(B->d_items, items.data(), sizeof(BItem) * items.size(), cudaMemcpyHostToDevice));
  B->nitems = (long)items.size();
  B->tile = tile;
  return IRIS_OK;
}

template <typename T, int TX, int TY, int TZ> int persistent_grid(const void* kern) {
  int nsm = 0, per = 0, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kern, TX * TY * TZ, 0);
  return std::max(1, nsm * std::max(1, per));
}

template <typename T, int TX, int TY, int TZ> void launch_batch_eh(iris_batch* B, bool e) {
  iris_engine* M = B->master;
  const dim3 blk(TX, TY, TZ);
  const FieldArgs<T>* args = (const FieldArgs<T>*)B->d_args;
  if (e) {
    static int grid = 0;
    if (!grid) grid = persistent_grid<T, TX, TY, TZ>((const void*)k_batch_e<T, TX, TY, TZ>);
    const long g = std::min<long>(grid, B->nitems);
    KTimer tm(M, IRIS_KC_E);
    k_batch_e<T, TX, TY, TZ><<<(unsigned)g, blk, 0, M->st>>>(args, B->d_items, B->nitems);
  } else {
    static int grid = 0;
    if (!grid) grid = persistent_grid<T, TX, TY, TZ>((const void*)k_batch_h<T, TX, TY, TZ>);
    const long g = std::min<long>(grid, B->nitems);
    KTimer tm(M, IRIS_KC_H);
    k_batch_h<T, TX, TY, TZ><<<(unsigned)g, blk, 0, M->st>>>(args, B->d_items, B->nitems);
  }
}

template <typename T, int MINB, bool CEPS, bool UPML>
void launch_flat_part(iris_batch* B, bool e, const BItem* items, long n) {
  if (n <= 0) return;
  iris_engine* M = B->master;
  const FieldArgs<T>* args = (const FieldArgs<T>*)B->d_args;
  auto kern = e ? k_batch_flat<T, true, MINB, CEPS, UPML> : k_batch_flat<T, false, MINB, false, UPML>;
  static int grid_e = 0, grid_h = 0;
  int& grid = e ? grid_e : grid_h;
  if (!grid) grid = persistent_grid<T, 256, 1, 1>((const void*)kern);
  kern<<<(unsigned)std::min<long>(grid, n), 256, 0, M->st>>>(args, items, n);
}

// One pass over a flat work list: the planes outside the UPML slabs with a
// kernel that has no slab code (fewer registers, more resident warps), then
// the slab planes.
template <typename T, int MINB, bool CEPS> void launch_flat(iris_batch* B, bool e) {
  KTimer tm(B->master, e ? IRIS_KC_E : IRIS_KC_H);
  launch_flat_part<T, MINB, CEPS, false>(B, e, B->d_items, B->nitems_in);
  launch_flat_part<T, MINB, CEPS, true>(B, e, B->d_items + B->nitems_in, B->nitems - B->nitems_in);
}

template <typename T, int MINB> void launch_batch_flat(iris_batch* B, bool e) {
  bool cplx = false;
  for (const iris_engine* E : B->cells) cplx |= E->eps_complex;
  if (cplx) launch_flat<T, MINB, true>(B, e);
  else launch_flat<T, MINB, false>(B, e);
}

template <typename T> void batch_eh(iris_batch* B, bool e) {
  switch (B->tile) {
    case FLAT: launch_batch_flat<T, 5>(B, e); break;
    case FLAT + 1: launch_batch_flat<T, 0>(B, e); break;
    case 0: launch_batch_eh<T, 32, 8, 1>(B, e); break;
    case 1: launch_batch_eh<T, 32, 4, 2>(B, e); break;
    case 2: launch_batch_eh<T, 64, 4, 1>(B, e); break;
    case 3: launch_batch_eh<T, 16, 16, 1>(B, e); break;
    default: launch_batch_eh<T, 32, 2, 4>(B, e); break;
  }
}

// One step of every cell: step it, or *itp + it when itp is given; sampled
// says whether the step's DFT sample is taken.
template <typename T> void batch_one_step(iris_batch* B, int it, const int* itp, bool sampled) {
  iris_engine* M = B->master;
  const iris_params& p = M->p;
  using V = typename V2<T>::t;
  const FieldArgs<T>* args = (const FieldArgs<T>*)B->d_args;
  batch_eh<T>(B, true);
  batch_eh<T>(B, false);
  if (B->ntitems) {
    KTimer tm(M, IRIS_KC_TFSF);
    const long g = std::min<long>(B->ntitems, 152L * 16);
    k_batch_tfsf<T><<<(unsigned)g, 64, 0, M->st>>>(args, B->d_src, B->d_titems, B->ntitems, it, itp);
  }
  if (sampled) {
    {
      KTimer tm(M, IRIS_KC_GATHER);
      V* slot = (V*)M->S + (long)M->nslot * M->P;
      dim3 grid((unsigned)((B->max_seg + 255) / 256), (unsigned)B->nbsegs);
      k_batch_gather<T><<<grid, 256, 0, M->st>>>(args, B->d_bsegs, slot, M->d_tk, M->nslot, it + 1 - p.to_fourier,
                                                 itp);
    }
    if (++M->nslot == M->K) dft_flush(M);
  }
}

template <typename T> int batch_step_t(iris_batch* B, int it0, int n) {
  iris_engine* M = B->master;
  const iris_params& p = M->p;
  int it = it0;
  while (it < it0 + n) {
    if (graph_ready(M, it, it0 + n - it)) {
      int rc = graph_block(M, it, [&] {
        for (int j = 0; j < M->K; ++j) batch_one_step<T>(B, j, M->d_it, true);
      });
      if (rc) return rc;
      it += M->K;
      continue;
    }
    batch_one_step<T>(B, it, nullptr, M->P > 0 && it >= p.to_fourier && it % p.sample_fourier == 0);
    ++it;
  }
  B->steps_taken += n;
  CK(cudaGetLastError());
  return IRIS_OK;
}

void batch_free(iris_batch* B) {
  for (iris_engine* E : B->cells)
    if (E) iris_destroy(E);
  void* ptrs[] = {B->d_args, B->d_src, B->d_items, B->d_titems, B->d_bsegs};
  for (void* q : ptrs)
    if (q) cudaFree(q);
  if (B->master) {
    free_engine(B->master);
    delete B->master;
  }
}

}  // namespace

extern "C" {

int iris_batch_create(int ncells, const iris_params* params, const double* fw, int dft_faces, iris_batch** out) {
  clear_error();
  if (ncells < 1 || !params || !fw || !out) return fail(IRIS_EINVAL, "bad argument");
  *out = nullptr;
  const iris_params& p0 = params[0];
  for (int c = 1; c < ncells; ++c) {
    const iris_params& q = params[c];
    if (q.precision != p0.precision || q.nof != p0.nof || q.dt != p0.dt || q.to_fourier != p0.to_fourier ||
        q.sample_fourier != p0.sample_fourier || q.device != p0.device || q.Q != p0.Q)
      return fail(IRIS_EINVAL, "batch cells must share precision, dt, Q, nof, DFT sampling and device");
  }
  if (p0.stencil == IRIS_STENCIL_FUSED) return fail(IRIS_EINVAL, "the batch steps with the split passes");
  iris_batch* B = new iris_batch();
  B->n = ncells;
  B->prec = p0.precision;
  B->device = p0.device;
  auto bail = [&](int code) {
    batch_free(B);
    delete B;
    return code;
  };
  B->cells.assign(ncells, nullptr);
  long P = 0;
  std::vector<BSeg> bsegs;
  std::vector<FluxFace> faces(6 * (size_t)ncells);
  std::vector<SrcArgs> srcs(ncells);
  std::vector<TItem> titems;
  for (int c = 0; c < ncells; ++c) {
    iris_params q = params[c];
    q.stencil = IRIS_STENCIL_SPLIT;
    int rc = create_engine(&q, fw, true, dft_faces == IRIS_DFT_Z, &B->cells[c], true);
    if (rc) return bail(rc);
    iris_engine* E = B->cells[c];
    B->pbase.push_back(P);
    for (const Seg& s : E->segs) {
      BSeg b{};
      b.s = s;
      b.s.p0 += P;
      b.cell = c;
      bsegs.push_back(b);
      B->max_seg = std::max(B->max_seg, (long)s.nu * s.nv);
    }
    for (int f = 0; f < 6; ++f) {
      FluxFace ff = E->host_faces[f];
      if (ff.active) {
        ff.pa += P;
        ff.pb += P;
        ff.pc += P;
        ff.pd += P;
      }
      faces[6 * c + f] = ff;
    }
    srcs[c] = E->src;
    if (E->src.variant != 0)
      for (int iy = 0; iy <= q.ny + 1; iy += TFSF_YCH)
        for (int ix = 0; ix <= q.nx + 1; ix += 64) titems.push_back(TItem{c, ix, iy, 0});
    P += E->P;
  }
  // the shell: one stream, the timers and the shared DFT buffers
  iris_engine* M = new iris_engine();
  B->master = M;
  M->p = params[0];
  M->fw.assign(fw, fw + p0.nof);
  M->prec = p0.precision;
  M->esz = p0.precision == IRIS_FP64 ? 16 : 8;
  M->device = p0.device;
  M->P = P;
  if (cudaSetDevice(M->device) != cudaSuccess) return bail(fail(IRIS_ECUDA, "cudaSetDevice failed"));
  if (cudaStreamCreateWithFlags(&M->st, cudaStreamNonBlocking) != cudaSuccess)
    return bail(fail(IRIS_ECUDA, "cudaStreamCreate failed"));
  int rc = alloc_dft(M, faces.data(), (int)faces.size());
  if (rc) return bail(rc);
  if (cudaMalloc(&B->d_bsegs, sizeof(BSeg) * std::max<size_t>(1, bsegs.size())) != cudaSuccess ||
      cudaMalloc(&B->d_src, sizeof(SrcArgs) * ncells) != cudaSuccess ||
      cudaMalloc(&B->d_titems, sizeof(TItem) * std::max<size_t>(1, titems.size())) != cudaSuccess)
    return bail(fail(IRIS_ENOMEM, "batch tables: allocation failed"));
  cudaMemcpy(B->d_bsegs, bsegs.data(), sizeof(BSeg) * bsegs.size(), cudaMemcpyHostToDevice);
  cudaMemcpy(B->d_src, srcs.data(), sizeof(SrcArgs) * ncells, cudaMemcpyHostToDevice);
  cudaMemcpy(B->d_titems, titems.data(), sizeof(TItem) * titems.size(), cudaMemcpyHostToDevice);
  B->nbsegs = (int)bsegs.size();
  B->ntitems = (long)titems.size();
  rc = batch_upload_args(B);
  if (rc) return bail(rc);
  rc = batch_build_items(B, 0);
  if (rc) return bail(rc);
  if (cudaStreamSynchronize(M->st) != cudaSuccess) return bail(fail(IRIS_ECUDA, "batch initialisation failed"));
  *out = B;
  return IRIS_OK;
}

void iris_batch_destroy(iris_batch* B) {
  if (!B) return;
  cudaSetDevice(B->device);
  if (B->master && B->master->st) cudaStreamSynchronize(B->master->st);
  batch_free(B);
  delete B;
}

int iris_batch_set_material(iris_batch* B, int cell, const double* re, const double* im) {
  clear_error();
  if (!B || cell < 0 || cell >= B->n) return fail(IRIS_EINVAL, "bad argument");
  CK(cudaSetDevice(B->device));
  CK(cudaStreamSynchronize(B->master->st));
  int rc = iris_set_material(B->cells[cell], re, im);
  if (rc) return rc;
  return batch_upload_args(B);  // the material pointer may have changed
}

int iris_batch_step(iris_batch* B, int it0, int nsteps) {
  clear_error();
  if (!B || nsteps < 0) return fail(IRIS_EINVAL, "bad argument");
  CK(cudaSetDevice(B->device));
  return B->prec == IRIS_FP64 ? batch_step_t<double>(B, it0, nsteps) : batch_step_t<float>(B, it0, nsteps);
}

int iris_batch_flux(iris_batch* B, int cell, double* J) {
  clear_error();
  if (!B || !J || cell < 0 || cell >= B->n) return fail(IRIS_EINVAL, "bad argument");
  CK(cudaSetDevice(B->device));
  iris_engine* M = B->master;
  const iris_params& p = M->p;
  dft_flush(M);
  const double scale = p.eps0 * p.Q / (2.0 * p.dt);
  k_flux<<<dim3(p.nof, 6), 256, 0, M->st>>>(M->fd, M->P, M->d_faces + 6 * cell, p.nof, scale, M->d_J);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(M->h_J, M->d_J, sizeof(double) * 6 * p.nof, cudaMemcpyDeviceToHost, M->st));
  CK(cudaStreamSynchronize(M->st));
  bool finite = true;
  for (int k = 0; k < 6 * p.nof; ++k) {
    J[k] = M->h_J[k];
    if (!std::isfinite(J[k])) finite = false;
  }
  return finite ? IRIS_OK : fail(IRIS_ENAN, "non-finite flux");
}

int iris_batch_get_field(iris_batch* B, int cell, int which, double* re, double* im) {
  clear_error();
  if (!B || cell < 0 || cell >= B->n) return fail(IRIS_EINVAL, "bad argument");
  CK(cudaSetDevice(B->device));
  CK(cudaStreamSynchronize(B->master->st));
  return iris_get_field(B->cells[cell], which, re, im);
}

int iris_batch_set_tile(iris_batch* B, int tile) {
  clear_error();
  if (!B || tile < 0 || tile >= NTILES) return fail(IRIS_EINVAL, "bad argument");
  CK(cudaSetDevice(B->device));
  CK(cudaStreamSynchronize(B->master->st));
  return batch_build_items(B, tile);
}

int iris_batch_tune(iris_batch* B, int reps, int* best, double* ms) {
  clear_error();
  if (!B || reps < 1) return fail(IRIS_EINVAL, "bad argument");
  if (B->steps_taken) return fail(IRIS_EINVAL, "tune before the first step (it runs E and H passes on the state)");
  CK(cudaSetDevice(B->device));
  iris_engine* M = B->master;
  cudaEvent_t a, b;
  CK(cudaEventCreate(&a));
  CK(cudaEventCreate(&b));
  int arg = 0;
  double bestms = 1e30;
  for (int t = 0; t < NTILES; ++t) {
    int rc = batch_build_items(B, t);
    if (rc) return rc;
    // fields are still zero, so E and H passes leave the state unchanged
    for (int r = 0; r < 2; ++r) {
      B->prec == IRIS_FP64 ? batch_eh<double>(B, true) : batch_eh<float>(B, true);
      B->prec == IRIS_FP64 ? batch_eh<double>(B, false) : batch_eh<float>(B, false);
    }
    CK(cudaEventRecord(a, M->st));
    for (int r = 0; r < reps; ++r) {
      B->prec == IRIS_FP64 ? batch_eh<double>(B, true) : batch_eh<float>(B, true);
      B->prec == IRIS_FP64 ? batch_eh<double>(B, false) : batch_eh<float>(B, false);
    }
    CK(cudaEventRecord(b, M->st));
    CK(cudaEventSynchronize(b));
    float x = 0;
    CK(cudaEventElapsedTime(&x, a, b));
    if (ms) ms[t] = x / reps;
    if (x < bestms) {
      bestms = x;
      arg = t;
    }
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (best) *best = arg;
  return batch_build_items(B, arg);
}

int iris_batch_timing(iris_batch* B, int enable) {
  if (!B) return fail(IRIS_EINVAL, "null batch");
  return iris_timing(B->master, enable);
}

int iris_batch_timing_read(iris_batch* B, double* region_ms, double* kernel_ms, long* launches) {
  if (!B) return fail(IRIS_EINVAL, "null batch");
  return iris_timing_read(B->master, region_ms, kernel_ms, launches);
}

int iris_batch_info(const iris_batch* B, long* info) {
  if (!B || !info) return fail(IRIS_EINVAL, "bad argument");
  long cells = 0;
  for (const iris_engine* E : B->cells) cells += (long)E->p.nx * E->p.ny * E->p.nz;
  info[0] = B->n;
  info[1] = cells;
  info[2] = B->master->P;
  info[3] = B->master->K;
  info[4] = B->tile;
  info[5] = B->nitems;
  info[6] = B->tile >= FLAT ? (B->nitems_in > 0) + (B->nitems > B->nitems_in) : 1;
  return IRIS_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Adjoint (gradient) form: the exact discrete adjoint of the time loop of
// code/driver.f90:338-451 as the engine runs it.
//
// One forward step maps the interior state (E, D, H, B; ghosts are Bloch
// images of interior cells) linearly, plus a TF/SF source that does not
// depend on the state:
//   E pass  D' = a D + b_e C,  E' = al E + g_e D + be_e C,   C  = curl_b H
//   H pass  B' = a B + b_h C', H' = al H + g_h B + be_h C',  C' = curl_f E'
// with, outside the UPML slabs, E' = E + m C (m = eps_inv, or 1/eps1, 1/eps3)
// and H' = H - dtcq2 C'.  Its conjugate transpose, applied in reverse order,
// uses curl_b^H = curl_f and curl_f^H = curl_b, whose Bloch ghosts carry the
// conjugated phase of the opposite side:
//   adjoint H pass  Ebar += curl_b(V),  V = b_h Bbar + be_h Hbar,
//                   then Hbar <- al Hbar, Bbar <- a Bbar + g_h Hbar
//   adjoint E pass  Hbar += curl_f(W),  W = b_e Dbar + be_e Ebar,
//                   then Ebar <- al Ebar, Dbar <- a Dbar + g_e Ebar
// Each "then" part touches one cell of a field whose neighbours the same
// kernel still reads, so it is deferred to the next kernel, which reads only
// its own cell of that field: both kernels update in place.
// dL/d eps_inv(c) = sum_n Re <Ebar'_n(c), C_n(c)>, Ebar'_n the adjoint of the
// E pass output of step n, C_n the forward curl of H that pass used.

namespace iris {
namespace {

// adjoint UPML rows, 24 per UPML plane (+k: component)
enum { AJ_A = 0, AJ_AL = 3, AJ_GE = 6, AJ_BE = 9, AJ_DE = 12, AJ_GH = 15, AJ_BH = 18, AJ_DH = 21 };

struct Design {
  int x0, y0, z0, nx, ny, nz;
  long n;
};

template <typename T> struct AdjArgs {
  FieldArgs<T> f;                // adjoint state; coef = adjoint rows, eps_r = forward material
  int z0;                        // first plane of the launch (blockIdx.z counts from it)
  int z1;                        // last plane of the launch
  Design d;
  const typename V2<T>::t* rec;  // forward curl of H at the design cells for this step, [3][n]
  double* grad;                  // dL/d eps_inv accumulators [n], or null
  int first;                     // no deferred E transform pending
};

struct AdjFace {
  long b[6];  // first sample index per component (Ex, Ey, Ez, Hx, Hy, Hz)
  long n;
  int nu, x0, y0, z;
};

template <typename T> __device__ __forceinline__ bool in_pml(const FieldArgs<T>& a, int z) {
  return z <= a.pmlzi || z >= a.pmlzf;
}

// UPML row and auxiliary index of interior cell (x, y, z) inside a slab.
template <typename T>
__device__ __forceinline__ void pml_at(const FieldArgs<T>& a, int x, int y, int z, int& slab, int& row, long& pi) {
  slab = z <= a.pmlzi ? 0 : 1;
  const int zr = slab == 0 ? z - 1 : z - a.pmlzf;
  row = slab == 0 ? z - 1 : a.pmlzi + z - a.pmlzf;
  pi = ((long)zr * a.g.ny + (y - 1)) * (long)a.g.nx + (x - 1);
}

// V_k = b_h Bbar_k + be_h Hbar_k (UPML) or -dtcq2 Hbar_k at interior cell
// (x, y, z); UPML = false: the caller knows z is outside the slabs.
template <typename T, bool UPML>
__device__ __forceinline__ cx<T> adj_v(const FieldArgs<T>& a, int x, int y, int z, int k) {
  const cx<T> hb = ld<T>(a.h + k * a.g.comp + a.g.at(x, y, z));
  if (UPML && in_pml(a, z)) {
    int slab, row;
    long pi;
    pml_at(a, x, y, z, slab, row, pi);
    const T* cf = a.coef + NCOEF * row;
    const cx<T> bb = ld<T>(a.pml_b[slab] + k * a.pcomp[slab] + pi);
    return cadd(rmul(cf[AJ_DH + k], bb), rmul(cf[AJ_BH + k], hb));
  }
  return rmul(-a.dtcq2, hb);
}

// W_k = b_e Dbar_k + be_e Ebar_k (UPML) or m Ebar_k at interior cell
// (x, y, z); UPML = false: the caller knows z is outside the slabs.
template <typename T, bool UPML>
__device__ __forceinline__ cx<T> adj_w(const FieldArgs<T>& a, int x, int y, int z, int k) {
  const Geo& g = a.g;
  const cx<T> eb = ld<T>(a.e + k * g.comp + g.at(x, y, z));
  if (UPML && in_pml(a, z)) {
    int slab, row;
    long pi;
    pml_at(a, x, y, z, slab, row, pi);
    const T* cf = a.coef + NCOEF * row;
    const cx<T> dd = ld<T>(a.pml_d[slab] + k * a.pcomp[slab] + pi);
    return cadd(rmul(cf[AJ_DE + k], dd), rmul(cf[AJ_BE + k], eb));
  }
  if (z >= a.hi && z <= a.hf) return rmul(a.eps_r[(long)(z - a.hi) * g.plane + (long)y * g.pitch + (x + g.xo)], eb);
  return rmul(z < a.hi ? a.m1 : a.m3, eb);
}

// Adjoint of the H pass (plus the E pass transform deferred from the step
// after it): Ebar += curl_b(V); the gradient term of the design cells.
// Planes z0 .. z1 of the launch; UPML = false: neither they nor the planes
// below them lie in a UPML slab.
template <typename T, bool CURL, bool UPML> __global__ void __launch_bounds__(256) k_adj_h(AdjArgs<T> A) {
  const FieldArgs<T>& a = A.f;
  const Geo& g = a.g;
  const int x = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int y = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int z = A.z0 + blockIdx.z * blockDim.z + threadIdx.z;
  if (x > g.nx || y > g.ny || z > A.z1) return;
  const long i = g.at(x, y, z);
  cx<T> e[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) e[k] = ld<T>(a.e + k * g.comp + i);
  if (UPML && !A.first && in_pml(a, z)) {
    int slab, row;
    long pi;
    pml_at(a, x, y, z, slab, row, pi);
    const T* cf = a.coef + NCOEF * row;
    auto* D = a.pml_d[slab];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const long j = k * a.pcomp[slab] + pi;
      st<T>(D + j, cadd(rmul(cf[AJ_A + k], ld<T>(D + j)), rmul(cf[AJ_GE + k], e[k])));
      e[k] = rmul(cf[AJ_AL + k], e[k]);
    }
  }
  if (CURL) {
    cx<T> v[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) v[k] = adj_v<T, UPML>(a, x, y, z, k);
    const int xm = x == 1 ? g.nx : x - 1, ym = y == 1 ? g.ny : y - 1, zm = z == 1 ? g.nz : z - 1;
    cx<T> v1x = adj_v<T, UPML>(a, xm, y, z, 1), v2x = adj_v<T, UPML>(a, xm, y, z, 2);
    cx<T> v0y = adj_v<T, UPML>(a, x, ym, z, 0), v2y = adj_v<T, UPML>(a, x, ym, z, 2);
    cx<T> v0z = adj_v<T, UPML>(a, x, y, zm, 0), v1z = adj_v<T, UPML>(a, x, y, zm, 1);
    if (x == 1) { v1x = cmul(a.pxm, v1x); v2x = cmul(a.pxm, v2x); }
    if (y == 1) { v0y = cmul(a.pym, v0y); v2y = cmul(a.pym, v2y); }
    if (z == 1) { v0z = cmul(a.pzm, v0z); v1z = cmul(a.pzm, v1z); }
    e[0] = cadd(e[0], cadd(csub(csub(v[2], v2y), v[1]), v1z));
    e[1] = cadd(e[1], cadd(csub(csub(v[0], v0z), v[2]), v2x));
    e[2] = cadd(e[2], cadd(csub(csub(v[1], v1x), v[0]), v0y));
    const Design& d = A.d;
    if (A.grad && x >= d.x0 && x < d.x0 + d.nx && y >= d.y0 && y < d.y0 + d.ny && z >= d.z0 && z < d.z0 + d.nz) {
      const long q = ((long)(z - d.z0) * d.ny + (y - d.y0)) * d.nx + (x - d.x0);
      T s = 0;
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const cx<T> c = ld<T>(A.rec + k * d.n + q);
        s = add_(s, add_(mul_(e[k].re, c.re), mul_(e[k].im, c.im)));
      }
      A.grad[q] += (double)s;
    }
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) st<T>(a.e + k * g.comp + i, e[k]);
}

// Adjoint of the E pass (plus the H pass transform of the same step):
// Hbar <- al Hbar + curl_f(W), Bbar <- a Bbar + g_h Hbar.  Planes z0 .. z1;
// UPML = false: neither they nor the planes above them lie in a UPML slab.
template <typename T, bool UPML> __global__ void __launch_bounds__(256) k_adj_e(AdjArgs<T> A) {
  const FieldArgs<T>& a = A.f;
  const Geo& g = a.g;
  const int x = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int y = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int z = A.z0 + blockIdx.z * blockDim.z + threadIdx.z;
  if (x > g.nx || y > g.ny || z > A.z1) return;
  const long i = g.at(x, y, z);
  cx<T> h[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) h[k] = ld<T>(a.h + k * g.comp + i);
  if (UPML && in_pml(a, z)) {
    int slab, row;
    long pi;
    pml_at(a, x, y, z, slab, row, pi);
    const T* cf = a.coef + NCOEF * row;
    auto* B = a.pml_b[slab];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const long j = k * a.pcomp[slab] + pi;
      st<T>(B + j, cadd(rmul(cf[AJ_A + k], ld<T>(B + j)), rmul(cf[AJ_GH + k], h[k])));
      h[k] = rmul(cf[AJ_AL + k], h[k]);
    }
  }
  cx<T> w[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) w[k] = adj_w<T, UPML>(a, x, y, z, k);
  const int xp = x == g.nx ? 1 : x + 1, yp = y == g.ny ? 1 : y + 1, zp = z == g.nz ? 1 : z + 1;
  cx<T> w1x = adj_w<T, UPML>(a, xp, y, z, 1), w2x = adj_w<T, UPML>(a, xp, y, z, 2);
  cx<T> w0y = adj_w<T, UPML>(a, x, yp, z, 0), w2y = adj_w<T, UPML>(a, x, yp, z, 2);
  cx<T> w0z = adj_w<T, UPML>(a, x, y, zp, 0), w1z = adj_w<T, UPML>(a, x, y, zp, 1);
  if (x == g.nx) { w1x = cmul(a.pxp, w1x); w2x = cmul(a.pxp, w2x); }
  if (y == g.ny) { w0y = cmul(a.pyp, w0y); w2y = cmul(a.pyp, w2y); }
  if (z == g.nz) { w0z = cmul(a.pzp, w0z); w1z = cmul(a.pzp, w1z); }
  h[0] = cadd(h[0], cadd(csub(csub(w2y, w[2]), w1z), w[1]));
  h[1] = cadd(h[1], cadd(csub(csub(w0z, w[0]), w2x), w[2]));
  h[2] = cadd(h[2], cadd(csub(csub(w1x, w[1]), w0y), w[0]));
#pragma unroll
  for (int k = 0; k < 3; ++k) st<T>(a.h + k * g.comp + i, h[k]);
}

// Forward curl_b H of the E pass at the design cells (the H the next E pass
// reads, ghosts included), as e_update forms it.
template <typename T>
__global__ void __launch_bounds__(256) k_adj_record(FieldArgs<T> a, Design d, typename V2<T>::t* __restrict__ rec) {
  const long q = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= d.n) return;
  const int x = d.x0 + (int)(q % d.nx), y = d.y0 + (int)((q / d.nx) % d.ny), z = d.z0 + (int)(q / ((long)d.nx * d.ny));
  const Geo& g = a.g;
  const long i = g.at(x, y, z);
  const auto* H1 = a.h;
  const auto* H2 = a.h + g.comp;
  const auto* H3 = a.h + 2 * g.comp;
  const cx<T> h0 = ld<T>(H1 + i), h1 = ld<T>(H2 + i), h2 = ld<T>(H3 + i);
  st<T>(rec + q, cadd(csub(csub(h2, ld<T>(H3 + i - g.pitch)), h1), ld<T>(H2 + i - g.plane)));
  st<T>(rec + d.n + q, cadd(csub(csub(h0, ld<T>(H1 + i - g.plane)), h2), ld<T>(H3 + i - 1)));
  st<T>(rec + 2 * d.n + q, cadd(csub(csub(h1, ld<T>(H2 + i - 1)), h0), ld<T>(H1 + i - g.pitch)));
}

// Adjoint DFT source of one sampled step on one z face:
//   Ebar_x += c Y_Hy, Ebar_y -= c Y_Hx, Hbar_x -= c Y_Ey, Hbar_y += c Y_Ex
// summed over frequencies, c = w * exp(-i fw t), Y the final DFT values.
template <typename T>
__global__ void __launch_bounds__(256) k_adj_source(typename V2<T>::t* __restrict__ ae, typename V2<T>::t* __restrict__ ah,
                                                    Geo g, const double2* __restrict__ fd, long P, AdjFace f,
                                                    const double* __restrict__ w, const double* __restrict__ fw,
                                                    int nof, int t) {
  extern __shared__ double2 tw[];
  for (int iw = threadIdx.x; iw < nof; iw += blockDim.x) {
    double s, c;
    sincos(fw[iw] * (double)t, &s, &c);
    tw[iw] = make_double2(w[iw] * c, -w[iw] * s);
  }
  __syncthreads();
  const long L = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (L >= f.n) return;
  double2 gex = {0, 0}, gey = {0, 0}, ghx = {0, 0}, ghy = {0, 0};
  for (int iw = 0; iw < nof; ++iw) {
    const double2* row = fd + (long)iw * P;
    const double2 xe = row[f.b[0] + L], ye = row[f.b[1] + L], xh = row[f.b[3] + L], yh = row[f.b[4] + L];
    const double2 c = tw[iw];
    gex.x += c.x * yh.x - c.y * yh.y; gex.y += c.x * yh.y + c.y * yh.x;
    ghy.x += c.x * xe.x - c.y * xe.y; ghy.y += c.x * xe.y + c.y * xe.x;
    gey.x -= c.x * xh.x - c.y * xh.y; gey.y -= c.x * xh.y + c.y * xh.x;
    ghx.x -= c.x * ye.x - c.y * ye.y; ghx.y -= c.x * ye.y + c.y * ye.x;
  }
  const long i = g.at(f.x0 + (int)(L % f.nu), f.y0 + (int)(L / f.nu), f.z);
  auto addv = [](typename V2<T>::t* p, double2 v) {
    typename V2<T>::t o = *p;
    o.x = (T)((double)o.x + v.x);
    o.y = (T)((double)o.y + v.y);
    *p = o;
  };
  addv(ae + i, gex);
  addv(ae + g.comp + i, gey);
  addv(ah + i, ghx);
  addv(ah + g.comp + i, ghy);
}

template <typename T> __global__ void k_adj_scatter(T* __restrict__ eps, Geo g, int hi, Design d, const T* __restrict__ v) {
  const long q = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= d.n) return;
  const int x = d.x0 + (int)(q % d.nx), y = d.y0 + (int)((q / d.nx) % d.ny), z = d.z0 + (int)(q / ((long)d.nx * d.ny));
  eps[(long)(z - hi) * g.plane + (long)y * g.pitch + (x + g.xo)] = v[q];
}

}  // namespace
}  // namespace iris

struct iris_adjoint {
  iris_engine* F = nullptr;  // forward engine (z-face DFT of box 1)
  iris_engine* A = nullptr;  // adjoint state: e, h, pml_d, pml_b
  void* acoef = nullptr;     // adjoint UPML rows
  Design d{};
  int K = 256;                 // checkpoint interval
  std::vector<double> w;       // [2][nof] objective weights
  double* d_w = nullptr;       // [2][nof] weight * sign * flux scale * dt
  bool side_on[2] = {false, false};
  double* d_grad = nullptr;    // [n]
  void* rec = nullptr;         // [K][3][n]
  int rec_seg = -1;            // segment whose curls rec holds
  void* d_design = nullptr;    // [n] staging for set_design
  std::vector<void*> ckpt;     // per segment: e, h, d0, d1, b0, b1
  size_t fbytes = 0, sbytes[2] = {0, 0};
  int nsteps = 0;
  double ms[3] = {0, 0, 0};
  cudaEvent_t ev[2] = {nullptr, nullptr};
};

namespace {

template <typename T> AdjArgs<T> adj_args(const iris_adjoint* J, bool first, int slot, bool grad) {
  AdjArgs<T> A{};
  A.f = field_args<T>(J->A);
  const FieldArgs<T> f = field_args<T>(J->F);
  A.f.coef = (const T*)J->acoef;
  A.f.eps_r = f.eps_r;
  A.f.eps_c = nullptr;
  auto conj = [](cx<T> c) { return cx<T>{c.re, -c.im}; };
  A.f.pxm = conj(f.pxp);
  A.f.pym = conj(f.pyp);
  A.f.pzm = conj(f.pzp);
  A.f.pxp = conj(f.pxm);
  A.f.pyp = conj(f.pym);
  A.f.pzp = conj(f.pzm);
  A.d = J->d;
  A.first = first ? 1 : 0;
  if (grad) {
    A.grad = J->d_grad;
    A.rec = (const typename V2<T>::t*)J->rec + (long)slot * 3 * J->d.n;
  }
  return A;
}

template <typename T> void adj_record(iris_adjoint* J, int slot) {
  iris_engine* F = J->F;
  using V = typename V2<T>::t;
  V* r = (V*)J->rec + (long)slot * 3 * J->d.n;
  k_adj_record<T><<<(unsigned)((J->d.n + 255) / 256), 256, 0, F->st>>>(field_args<T>(F), J->d, r);
}

template <typename T> void adj_source(iris_adjoint* J, int t) {
  iris_engine* F = J->F;
  const FaceMap& M = F->fm[0][2];
  const iris_params& p = F->p;
  using V = typename V2<T>::t;
  for (int side = 0; side < 2; ++side) {
    if (!J->side_on[side]) continue;
    AdjFace f{};
    for (int c = 0; c < 6; ++c) f.b[c] = M.base[side][c];
    f.n = M.nloc;
    f.nu = M.nu;
    f.x0 = p.box1[0];
    f.y0 = p.box1[2];
    f.z = side == 0 ? p.box1[4] : p.box1[5];
    k_adj_source<T><<<(unsigned)((f.n + 255) / 256), 256, sizeof(double2) * p.nof, F->st>>>(
        (V*)J->A->e, (V*)J->A->h, F->g, F->fd, F->P, f, J->d_w + side * p.nof, F->d_fw, p.nof, t);
  }
}

// Launch shape of planes z0 .. z1 (none when z1 < z0).
dim3 adj_grid(const iris_engine* F, int z0, int z1) {
  return dim3(F->grd.x, F->grd.y, z1 < z0 ? 0u : (unsigned)((z1 - z0 + F->blk.z) / F->blk.z));
}

// One adjoint step (K1 then K2) for forward step it; rec slot or -1.  Each
// kernel runs as the planes whose stencil stays outside the UPML slabs,
// compiled without slab code, and the rest (the slabs and their neighbours).
template <typename T> void adj_step(iris_adjoint* J, bool first, int slot) {
  iris_engine* F = J->F;
  const iris_params& p = F->p;
  const bool grad = slot >= 0;
  AdjArgs<T> a = adj_args<T>(J, first, slot, grad);
  auto k1 = [&](int z0, int z1, bool upml) {
    a.z0 = z0;
    a.z1 = z1;
    const dim3 gr = adj_grid(F, z0, z1);
    if (gr.z == 0) return;
    if (upml) k_adj_h<T, true, true><<<gr, F->blk, 0, F->st>>>(a);
    else k_adj_h<T, true, false><<<gr, F->blk, 0, F->st>>>(a);
  };
  // K1 reads planes z and z-1: free of slab code for z in [pmlzi+2, pmlzf-1]
  const int a1 = std::min(p.pmlzi + 1, p.pmlzf - 1);
  k1(1, a1, true);
  k1(a1 + 1, p.pmlzf - 1, false);
  k1(p.pmlzf, p.nz, true);
  AdjArgs<T> b = adj_args<T>(J, first, -1, false);
  auto k2 = [&](int z0, int z1, bool upml) {
    b.z0 = z0;
    b.z1 = z1;
    const dim3 gr = adj_grid(F, z0, z1);
    if (gr.z == 0) return;
    if (upml) k_adj_e<T, true><<<gr, F->blk, 0, F->st>>>(b);
    else k_adj_e<T, false><<<gr, F->blk, 0, F->st>>>(b);
  };
  // K2 reads planes z and z+1: free of slab code for z in [pmlzi+1, pmlzf-2]
  const int b2 = std::max(p.pmlzf - 2, p.pmlzi);
  k2(1, p.pmlzi, true);
  k2(p.pmlzi + 1, b2, false);
  k2(b2 + 1, p.nz, true);
}

template <typename T> void adj_finalize(iris_adjoint* J) {
  iris_engine* F = J->F;
  AdjArgs<T> a = adj_args<T>(J, false, -1, false);
  a.z0 = 1;
  a.z1 = F->p.nz;
  k_adj_h<T, false, true><<<adj_grid(F, 1, F->p.nz), F->blk, 0, F->st>>>(a);
}

// The forward step without DFT sampling (recompute) or with it (forward).
template <typename T> void fwd_step(iris_engine* F, int it, bool dft) {
  launch_e<T>(F);
  launch_h<T>(F);
  launch_tfsf<T>(F, it);
  const iris_params& p = F->p;
  if (dft && it >= p.to_fourier && it % p.sample_fourier == 0) dft_sample<T>(F, it + 1 - p.to_fourier);
}

int ckpt_io(iris_adjoint* J, int seg, bool save) {
  iris_engine* F = J->F;
  unsigned char* c = (unsigned char*)J->ckpt[seg];
  void* parts[6] = {F->e, F->h, F->pml_d[0], F->pml_d[1], F->pml_b[0], F->pml_b[1]};
  const size_t sz[6] = {J->fbytes, J->fbytes, J->sbytes[0], J->sbytes[1], J->sbytes[0], J->sbytes[1]};
  size_t off = 0;
  for (int k = 0; k < 6; ++k) {
    if (save) CK(cudaMemcpyAsync(c + off, parts[k], sz[k], cudaMemcpyDeviceToDevice, F->st));
    else CK(cudaMemcpyAsync(parts[k], c + off, sz[k], cudaMemcpyDeviceToDevice, F->st));
    off += sz[k];
  }
  return IRIS_OK;
}

int zero_state(iris_engine* E, size_t fbytes, const size_t* sbytes) {
  CK(cudaMemsetAsync(E->e, 0, fbytes, E->st));
  CK(cudaMemsetAsync(E->h, 0, fbytes, E->st));
  for (int s = 0; s < 2; ++s) {
    CK(cudaMemsetAsync(E->pml_d[s], 0, sbytes[s], E->st));
    CK(cudaMemsetAsync(E->pml_b[s], 0, sbytes[s], E->st));
  }
  return IRIS_OK;
}

template <typename T> int adj_forward(iris_adjoint* J, int nsteps) {
  iris_engine* F = J->F;
  const int S = (nsteps + J->K - 1) / J->K;
  const size_t cbytes = 2 * J->fbytes + 2 * (J->sbytes[0] + J->sbytes[1]);
  while ((int)J->ckpt.size() < S) {
    void* q = nullptr;
    if (cudaMalloc(&q, cbytes) != cudaSuccess) {
      cudaGetLastError();
      return fail(IRIS_ENOMEM, "checkpoint allocation failed (" + std::to_string(S) + " checkpoints of " +
                                   std::to_string(cbytes) + " bytes)");
    }
    J->ckpt.push_back(q);
  }
  int rc = zero_state(F, J->fbytes, J->sbytes);
  if (rc) return rc;
  CK(cudaMemsetAsync(F->fd, 0, (size_t)F->P * F->p.nof * sizeof(double2), F->st));
  F->nslot = 0;
  CK(cudaEventRecord(J->ev[0], F->st));
  for (int it = 1; it <= nsteps; ++it) {
    const int seg = (it - 1) / J->K;
    if ((it - 1) % J->K == 0) {
      rc = ckpt_io(J, seg, true);
      if (rc) return rc;
    }
    if (seg == S - 1) adj_record<T>(J, it - 1 - seg * J->K);
    fwd_step<T>(F, it, true);
  }
  dft_flush(F);
  CK(cudaEventRecord(J->ev[1], F->st));
  CK(cudaEventSynchronize(J->ev[1]));
  float x = 0.f;
  CK(cudaEventElapsedTime(&x, J->ev[0], J->ev[1]));
  J->ms[0] = x;
  J->rec_seg = S - 1;
  J->nsteps = nsteps;
  CK(cudaGetLastError());
  return IRIS_OK;
}

template <typename T> int adj_backward(iris_adjoint* J) {
  iris_engine* F = J->F;
  const iris_params& p = F->p;
  const int N = J->nsteps, S = (N + J->K - 1) / J->K;
  int rc = zero_state(J->A, J->fbytes, J->sbytes);
  if (rc) return rc;
  CK(cudaMemsetAsync(J->d_grad, 0, sizeof(double) * J->d.n, F->st));
  double t_rec = 0, t_adj = 0;
  bool first = true;
  for (int seg = S - 1; seg >= 0; --seg) {
    const int s0 = seg * J->K + 1, s1 = std::min(N, (seg + 1) * J->K);
    float x = 0.f;
    if (J->rec_seg != seg) {
      CK(cudaEventRecord(J->ev[0], F->st));
      rc = ckpt_io(J, seg, false);
      if (rc) return rc;
      for (int it = s0; it <= s1; ++it) {
        adj_record<T>(J, it - s0);
        fwd_step<T>(F, it, false);
      }
      CK(cudaEventRecord(J->ev[1], F->st));
      CK(cudaEventSynchronize(J->ev[1]));
      CK(cudaEventElapsedTime(&x, J->ev[0], J->ev[1]));
      t_rec += x;
      J->rec_seg = seg;
    }
    CK(cudaEventRecord(J->ev[0], F->st));
    for (int it = s1; it >= s0; --it) {
      if (it >= p.to_fourier && it % p.sample_fourier == 0) adj_source<T>(J, it + 1 - p.to_fourier);
      adj_step<T>(J, first, it - s0);
      first = false;
    }
    CK(cudaEventRecord(J->ev[1], F->st));
    CK(cudaEventSynchronize(J->ev[1]));
    CK(cudaEventElapsedTime(&x, J->ev[0], J->ev[1]));
    t_adj += x;
  }
  J->ms[1] = t_rec;
  J->ms[2] = t_adj;
  CK(cudaGetLastError());
  return IRIS_OK;
}

void adj_free(iris_adjoint* J) {
  if (J->F) iris_destroy(J->F);
  if (J->A) iris_destroy(J->A);
  void* ptrs[] = {J->acoef, J->d_w, J->d_grad, J->rec, J->d_design};
  for (void* q : ptrs)
    if (q) cudaFree(q);
  for (void* q : J->ckpt)
    if (q) cudaFree(q);
  for (cudaEvent_t e : J->ev)
    if (e) cudaEventDestroy(e);
}

}  // namespace

extern "C" {

int iris_adjoint_create(const iris_params* pin, const double* fw, const int design[6], int checkpoint_every,
                        const double* weights, iris_adjoint** out) {
  clear_error();
  if (!pin || !fw || !design || !out) return fail(IRIS_EINVAL, "null argument");
  *out = nullptr;
  const iris_params& p = *pin;
  if (checkpoint_every < 1) return fail(IRIS_EINVAL, "checkpoint_every must be >= 1");
  const int* D = design;
  if (D[0] < 1 || D[1] > p.nx || D[0] > D[1] || D[2] < 1 || D[3] > p.ny || D[2] > D[3] || D[4] < p.hi ||
      D[5] > p.hf || D[4] > D[5])
    return fail(IRIS_EINVAL, "design region must lie in [1,nx] x [1,ny] x [hi,hf]");
  if (p.hi <= p.pmlzi || p.hf >= p.pmlzf) return fail(IRIS_EINVAL, "the structure layer must lie outside the UPML slabs");
  if (p.box1[4] <= p.pmlzi || p.box1[5] >= p.pmlzf)
    return fail(IRIS_EINVAL, "the DFT z planes of box 1 must lie outside the UPML slabs");
  iris_adjoint* J = new iris_adjoint();
  auto bail = [&](int code) {
    adj_free(J);
    delete J;
    return code;
  };
  iris_params q = p;
  q.stencil = IRIS_STENCIL_SPLIT;
  for (int i = 0; i < 6; ++i) q.box2[i] = q.box1[i];
  int rc = create_engine(&q, fw, false, true, &J->F);
  if (rc) return bail(rc);
  rc = create_engine(&q, fw, true, true, &J->A);
  if (rc) return bail(rc);
  iris_engine* F = J->F;
  J->K = checkpoint_every;
  J->d = Design{D[0], D[2], D[4], D[1] - D[0] + 1, D[3] - D[2] + 1, D[5] - D[4] + 1, 0};
  J->d.n = (long)J->d.nx * J->d.ny * J->d.nz;
  J->fbytes = (size_t)3 * F->g.comp * F->esz;
  for (int s = 0; s < 2; ++s) J->sbytes[s] = (size_t)3 * F->pcomp[s] * F->esz;
  // objective weights, folded with the flux sign and scale and the DFT's dt
  const int nof = p.nof;
  J->w.assign(2 * (size_t)nof, 0.0);
  for (int k = 0; k < nof; ++k) J->w[nof + k] = 1.0;
  if (weights) J->w.assign(weights, weights + 2 * nof);
  std::vector<double> wd(2 * (size_t)nof);
  const double scale = p.eps0 * p.Q / (2.0 * p.dt);
  for (int side = 0; side < 2; ++side)
    for (int k = 0; k < nof; ++k) {
      const double v = J->w[side * nof + k];
      wd[side * nof + k] = (side == 0 ? -1.0 : 1.0) * scale * p.dt * v;
      if (v != 0.0) J->side_on[side] = true;
    }
  // adjoint UPML rows from the forward ones
  const std::vector<double>& c = F->coef_h;
  const size_t nrow = c.size() / NCOEF;
  std::vector<double> ac(c.size());
  const double e2 = p.eps0 * p.eps0;
  for (size_t r = 0; r < nrow; ++r) {
    const double* f = c.data() + NCOEF * r;
    double* a = ac.data() + NCOEF * r;
    for (int k = 0; k < 3; ++k) {
      a[AJ_A + k] = f[CD_A + k];
      a[AJ_AL + k] = f[CE_A + k];
      a[AJ_GE + k] = f[CE_B + k] * (f[C_FP + k] * f[CD_A + k] - f[C_FM + k]);
      a[AJ_BE + k] = f[CE_B + k] * f[C_FP + k] * f[CD_B + k] * e2;
      a[AJ_DE + k] = f[CD_B + k] * e2;
      a[AJ_GH + k] = f[CH_B + k] * (f[C_FP + k] * f[CD_A + k] - f[C_FM + k]);
      a[AJ_BH + k] = -f[CH_B + k] * f[C_FP + k] * f[CB_B + k];
      a[AJ_DH + k] = -f[CB_B + k];
    }
  }
  const size_t rsz = F->prec == IRIS_FP64 ? 8 : 4;
  const size_t csz = F->prec == IRIS_FP64 ? 16 : 8;
  auto dev_alloc = [&](void** q2, size_t b) { return cudaMalloc(q2, std::max<size_t>(b, 16)) == cudaSuccess; };
  if (!dev_alloc(&J->acoef, ac.size() * rsz) || !dev_alloc((void**)&J->d_w, sizeof(double) * 2 * nof) ||
      !dev_alloc((void**)&J->d_grad, sizeof(double) * J->d.n) ||
      !dev_alloc(&J->rec, (size_t)J->K * 3 * J->d.n * csz) || !dev_alloc(&J->d_design, J->d.n * rsz)) {
    cudaGetLastError();
    return bail(fail(IRIS_ENOMEM, "adjoint buffers: allocation failed"));
  }
  if (F->prec == IRIS_FP64) {
    if (cudaMemcpy(J->acoef, ac.data(), ac.size() * 8, cudaMemcpyHostToDevice) != cudaSuccess)
      return bail(fail(IRIS_ECUDA, "adjoint rows upload failed"));
  } else {
    std::vector<float> af(ac.begin(), ac.end());
    if (cudaMemcpy(J->acoef, af.data(), af.size() * 4, cudaMemcpyHostToDevice) != cudaSuccess)
      return bail(fail(IRIS_ECUDA, "adjoint rows upload failed"));
  }
  if (cudaMemcpy(J->d_w, wd.data(), sizeof(double) * 2 * nof, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaEventCreate(&J->ev[0]) != cudaSuccess || cudaEventCreate(&J->ev[1]) != cudaSuccess)
    return bail(fail(IRIS_ECUDA, "adjoint initialisation failed"));
  *out = J;
  return IRIS_OK;
}

void iris_adjoint_destroy(iris_adjoint* J) {
  if (!J) return;
  cudaSetDevice(J->F ? J->F->device : 0);
  if (J->F) cudaStreamSynchronize(J->F->st);
  adj_free(J);
  delete J;
}

int iris_adjoint_set_material(iris_adjoint* J, const double* re, const double* im) {
  clear_error();
  if (!J || !re) return fail(IRIS_EINVAL, "null argument");
  int rc = iris_set_material(J->F, re, im);
  if (rc) return rc;
  if (J->F->eps_complex) return fail(IRIS_EINVAL, "the adjoint form needs a real material");
  return IRIS_OK;
}

int iris_adjoint_set_design(iris_adjoint* J, const double* v) {
  clear_error();
  if (!J || !v) return fail(IRIS_EINVAL, "null argument");
  iris_engine* F = J->F;
  CK(cudaSetDevice(F->device));
  if (F->eps_complex) return fail(IRIS_EINVAL, "the adjoint form needs a real material");
  const unsigned nb = (unsigned)((J->d.n + 255) / 256);
  if (F->prec == IRIS_FP64) {
    CK(cudaMemcpyAsync(J->d_design, v, sizeof(double) * J->d.n, cudaMemcpyHostToDevice, F->st));
    k_adj_scatter<double><<<nb, 256, 0, F->st>>>((double*)F->eps, F->g, F->p.hi, J->d, (const double*)J->d_design);
  } else {
    std::vector<float> f(v, v + J->d.n);
    CK(cudaMemcpyAsync(J->d_design, f.data(), sizeof(float) * J->d.n, cudaMemcpyHostToDevice, F->st));
    k_adj_scatter<float><<<nb, 256, 0, F->st>>>((float*)F->eps, F->g, F->p.hi, J->d, (const float*)J->d_design);
  }
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(F->st));
  return IRIS_OK;
}

int iris_adjoint_forward(iris_adjoint* J, int nsteps, double* L, double* Jout) {
  clear_error();
  if (!J || nsteps < 1) return fail(IRIS_EINVAL, "bad argument");
  iris_engine* F = J->F;
  CK(cudaSetDevice(F->device));
  if (F->eps_complex) return fail(IRIS_EINVAL, "the adjoint form needs a real material");
  int rc = F->prec == IRIS_FP64 ? adj_forward<double>(J, nsteps) : adj_forward<float>(J, nsteps);
  if (rc) return rc;
  const int nof = F->p.nof;
  std::vector<double> flux(6 * (size_t)nof);
  rc = iris_flux(F, 0, flux.data());
  if (rc) return rc;
  double s = 0.0;
  for (int k = 0; k < nof; ++k) s += J->w[k] * flux[4 * nof + k] + J->w[nof + k] * flux[5 * nof + k];
  if (L) *L = s;
  if (Jout) std::copy(flux.begin(), flux.end(), Jout);
  return IRIS_OK;
}

int iris_adjoint_backward(iris_adjoint* J, double* grad) {
  clear_error();
  if (!J || !grad) return fail(IRIS_EINVAL, "null argument");
  if (J->nsteps < 1) return fail(IRIS_EINVAL, "no forward solve to differentiate");
  iris_engine* F = J->F;
  CK(cudaSetDevice(F->device));
  int rc = F->prec == IRIS_FP64 ? adj_backward<double>(J) : adj_backward<float>(J);
  if (rc) return rc;
  CK(cudaMemcpyAsync(grad, J->d_grad, sizeof(double) * J->d.n, cudaMemcpyDeviceToHost, F->st));
  CK(cudaStreamSynchronize(F->st));
  for (long q = 0; q < J->d.n; ++q)
    if (!std::isfinite(grad[q])) return fail(IRIS_ENAN, "non-finite gradient");
  return IRIS_OK;
}

int iris_adjoint_engine(iris_adjoint* J, int which, iris_engine** eng) {
  if (!J || !eng || (which != 0 && which != 1)) return fail(IRIS_EINVAL, "bad argument");
  *eng = which == 0 ? J->F : J->A;
  return IRIS_OK;
}

int iris_adjoint_apply(iris_adjoint* J, int nsteps) {
  clear_error();
  if (!J || nsteps < 0) return fail(IRIS_EINVAL, "bad argument");
  iris_engine* F = J->F;
  CK(cudaSetDevice(F->device));
  CK(cudaStreamSynchronize(J->A->st));
  const bool d = F->prec == IRIS_FP64;
  for (int k = 0; k < nsteps; ++k) d ? adj_step<double>(J, k == 0, -1) : adj_step<float>(J, k == 0, -1);
  if (nsteps > 0) d ? adj_finalize<double>(J) : adj_finalize<float>(J);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(F->st));
  return IRIS_OK;
}

int iris_adjoint_timing(const iris_adjoint* J, double* ms) {
  if (!J || !ms) return fail(IRIS_EINVAL, "bad argument");
  for (int k = 0; k < 3; ++k) ms[k] = J->ms[k];
  return IRIS_OK;
}

}  // extern "C"
