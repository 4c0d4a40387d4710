// Device types and per-cell operators shared by the engine, batched and
// adjoint kernels: complex arithmetic in both precisions, the grid geometry,
// the E/H cell updates with their UPML and Bloch-ghost forms, the TF/SF
// incident field, the DFT point runs and the flux faces.  Not part of the
// public ABI.
//
// Arithmetic: the FP64 mode uses __dmul_rn/__dadd_rn (never contracted to
// FMA) so the stencil rounds exactly like the reference build; the FP32 mode
// lets the compiler contract.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

namespace iris {

// ---------------------------------------------------------------------------
// Bounds checks (built with -DIRIS_BOUNDS_CHECK: libiris_fdtd_bc.so).  At the
// points where a kernel maps its thread to a cell, a slab row, a correction
// row, a DFT point or an accumulator, bc_ok tests the index against its
// range; the first failure of the process's kernels is recorded as
// (site << 48) | (index & 0xffffffffffff) in a device word of the module and
// the access is skipped.  iris_bounds_check reads and clears the words.  In
// the ordinary build bc_ok is the constant true and costs nothing.
enum BcSite {
  BC_E_CELL = 1, BC_H_CELL, BC_E_SLAB, BC_H_SLAB, BC_EPS, BC_TFSF, BC_GATHER_SRC, BC_GATHER_DST,
  BC_FUSED_CELL, BC_FUSED_SLAB, BC_DFT_POINT, BC_DFT_SAMPLE, BC_FLUX_POINT
};
#ifdef IRIS_BOUNDS_CHECK
static __device__ unsigned long long g_bc_first;
__device__ __forceinline__ bool bc_ok(bool ok, int site, long v) {
  if (!ok) atomicCAS(&g_bc_first, 0ull, ((unsigned long long)site << 48) | ((unsigned long long)v & 0xffffffffffffull));
  return ok;
}
// The module's record, cleared (host).
static inline unsigned long long bc_take_module() {
  unsigned long long v = 0, z = 0;
  if (cudaMemcpyFromSymbol(&v, g_bc_first, sizeof v) != cudaSuccess) return ~0ull;
  cudaMemcpyToSymbol(g_bc_first, &z, sizeof z);
  return v;
}
#else
__device__ __forceinline__ bool bc_ok(bool, int, long) { return true; }
static inline unsigned long long bc_take_module() { return 0; }
#endif

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

__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

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
// cell lies outside the UPML slabs (the slab code is not compiled in).  A
// caller that has copied the cell's old D (dv, 3 values) or the plane's
// coefficient row (cfv) ahead passes them instead of their global copies.
template <typename T, bool CEPS, int MASK = 7, bool EPV = false, bool UPML = true>
__device__ __forceinline__ void e_apply(const FieldArgs<T>& a, typename V2<T>::t* const* dnew, int x, int y, int z,
                                        const cx<T> c[3], cx<T> e[3], T ep = T(0), const cx<T>* dv = nullptr,
                                        const T* cfv = nullptr) {
  using V = typename V2<T>::t;
  const Geo& g = a.g;
  if (UPML && (z <= a.pmlzi || z >= a.pmlzf)) {
    const int slab = z <= a.pmlzi ? 0 : 1;
    const int zr = slab == 0 ? z - 1 : z - a.pmlzf;
    const int row = slab == 0 ? z - 1 : a.pmlzi + z - a.pmlzf;
    const T* cf = cfv ? cfv : a.coef + NCOEF * row;
    const long pi = ((long)zr * g.ny + (y - 1)) * (long)g.nx + (x - 1);
    const V* D = a.pml_d[slab];
    const long pc = a.pcomp[slab];
    if (!bc_ok(pi >= 0 && pi < pc, BC_E_SLAB, pi)) return;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      if (!(MASK & (1 << k))) continue;
      const cx<T> ck = rmul(a.eps0sq, c[k]);
      const cx<T> dold = dv ? dv[k] : ld<T>(D + k * pc + pi);
      const cx<T> dn = cadd(rmul(cf[CD_A + k], dold), rmul(cf[CD_B + k], ck));
      if (dnew) st<T>(dnew[slab] + k * pc + pi, dn);
      e[k] = cadd(rmul(cf[CE_A + k], e[k]), rmul(cf[CE_B + k], csub(rmul(cf[C_FP + k], dn), rmul(cf[C_FM + k], dold))));
    }
  } else if (z >= a.hi && z <= a.hf) {
    const long ie = (long)(z - a.hi) * g.plane + (long)y * g.pitch + (long)(x + g.xo);
    if (!bc_ok(x >= 0 && x <= g.nx + 1 && y >= 0 && y <= g.ny + 1, BC_EPS, ie)) return;
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
// false: the cell lies outside the UPML slabs.  bv / cfv: the cell's old B and
// the plane's coefficient row when the caller has copied them ahead.  MASK
// selects the components computed (bit k: H_{k+1}).
template <typename T, bool UPML = true, int MASK = 7>
__device__ __forceinline__ void h_update(const FieldArgs<T>& a, int x, int y, int z, const cx<T> ev[3],
                                         const cx<T> xp[3], const cx<T> yp[3], const cx<T> zp[3], cx<T> h[3],
                                         const cx<T>* bv = nullptr, const T* cfv = nullptr) {
  using V = typename V2<T>::t;
  const Geo& g = a.g;
  cx<T> c[3];
  if (MASK & 1) c[0] = cadd(csub(csub(yp[2], ev[2]), zp[1]), ev[1]);
  if (MASK & 2) c[1] = cadd(csub(csub(zp[0], ev[0]), xp[2]), ev[2]);
  if (MASK & 4) c[2] = cadd(csub(csub(xp[1], ev[1]), yp[0]), ev[0]);
  if (UPML && (z <= a.pmlzi || z >= a.pmlzf)) {
    const int slab = z <= a.pmlzi ? 0 : 1;
    const int zr = slab == 0 ? z - 1 : z - a.pmlzf;
    const int row = slab == 0 ? z - 1 : a.pmlzi + z - a.pmlzf;
    const T* cf = cfv ? cfv : a.coef + NCOEF * row;
    const long pi = ((long)zr * g.ny + (y - 1)) * (long)g.nx + (x - 1);
    V* B = a.pml_b[slab];
    const long pc = a.pcomp[slab];
    if (!bc_ok(pi >= 0 && pi < pc, BC_H_SLAB, pi)) return;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      if (!(MASK & (1 << k))) continue;
      const cx<T> bold = bv ? bv[k] : ld<T>(B + k * pc + pi);
      const cx<T> bn = csub(rmul(cf[CD_A + k], bold), rmul(cf[CB_B + k], c[k]));
      st<T>(B + k * pc + pi, bn);
      h[k] = cadd(rmul(cf[CE_A + k], h[k]), rmul(cf[CH_B + k], csub(rmul(cf[C_FP + k], bn), rmul(cf[C_FM + k], bold))));
    }
  } else {
#pragma unroll
    for (int k = 0; k < 3; ++k)
      if (MASK & (1 << k)) h[k] = csub(h[k], rmul(a.dtcq2, c[k]));
  }
}

// h_update with the old H of the cell loaded from a.h.
template <typename T, bool UPML = true, int MASK = 7>
__device__ __forceinline__ void h_cell(const FieldArgs<T>& a, int x, int y, int z, const cx<T> ev[3],
                                       const cx<T> xp[3], const cx<T> yp[3], const cx<T> zp[3], cx<T> h[3]) {
  const long i = a.g.at(x, y, z);
#pragma unroll
  for (int k = 0; k < 3; ++k)
    if (MASK & (1 << k)) h[k] = ld<T>(a.h + k * a.g.comp + i);
  h_update<T, UPML, MASK>(a, x, y, z, ev, xp, yp, zp, h);
}

// Split E pass of one cell: e_cell in place + bc_{x,y,z}max_bloch
// (code/boundary.f90:193-216,257-284,321-348) for the E ghosts.  MASK: the
// components computed and stored (bit k: E_{k+1}); the components of a cell
// are independent, so a cell may be split over threads.
template <typename T, bool CEPS, bool UPML = true, int MASK = 7>
__device__ __forceinline__ void e_split_cell(const FieldArgs<T>& a, int x, int y, int z) {
  using V = typename V2<T>::t;
  const Geo& g = a.g;
  const long i = g.at(x, y, z);
  if (!bc_ok(x >= 1 && x <= g.nx && y >= 1 && y <= g.ny && z >= 1 && z <= g.nz, BC_E_CELL, i)) return;
  V* E[3] = {a.e, a.e + g.comp, a.e + 2 * g.comp};
  cx<T> e[3];
  e_cell<T, CEPS, MASK, UPML>(a, a.pml_d, x, y, z, e);
#pragma unroll
  for (int k = 0; k < 3; ++k)
    if (MASK & (1 << k)) st<T>(E[k] + i, e[k]);
  if (x == 1) {
    const long j = g.at(g.nx + 1, y, z);
#pragma unroll
    for (int k = 0; k < 3; ++k)
      if (MASK & (1 << k)) st<T>(E[k] + j, cmul(a.pxp, e[k]));
  }
  if (y == 1) {
    const long j = g.at(x, g.ny + 1, z);
#pragma unroll
    for (int k = 0; k < 3; ++k)
      if (MASK & (1 << k)) st<T>(E[k] + j, cmul(a.pyp, e[k]));
  }
  if (z == 1) {
    const long j = g.at(x, y, g.nz + 1);
#pragma unroll
    for (int k = 0; k < 3; ++k)
      if (MASK & (1 << k)) st<T>(E[k] + j, cmul(a.pzp, e[k]));
  }
}

// Split H pass of one cell: h_cell in place + bc_{x,y,z}min_bloch
// (code/boundary.f90:163-187,224-251,288-315) for the H ghosts and the E
// ghosts at 0.  The ghosts at nx+1/ny+1/nz+1 of H are never read by any
// operator and are not maintained.
template <typename T, bool UPML = true, int MASK = 7>
__device__ __forceinline__ void h_split_cell(const FieldArgs<T>& a, int x, int y, int z) {
  using V = typename V2<T>::t;
  const Geo& g = a.g;
  const long i = g.at(x, y, z);
  if (!bc_ok(x >= 1 && x <= g.nx && y >= 1 && y <= g.ny && z >= 1 && z <= g.nz, BC_H_CELL, i)) return;
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
  h_cell<T, UPML, MASK>(a, x, y, z, ev, xp, yp, zp, h);
#pragma unroll
  for (int k = 0; k < 3; ++k)
    if (MASK & (1 << k)) st<T>(H[k] + i, h[k]);
  if (x == g.nx) {
    const long j = g.at(0, y, z);
#pragma unroll
    for (int k = 0; k < 3; ++k)
      if (MASK & (1 << k)) {
        st<T>(Ec[k] + j, cmul(a.pxm, ev[k]));
        st<T>(H[k] + j, cmul(a.pxm, h[k]));
      }
  }
  if (y == g.ny) {
    const long j = g.at(x, 0, z);
#pragma unroll
    for (int k = 0; k < 3; ++k)
      if (MASK & (1 << k)) {
        st<T>(Ec[k] + j, cmul(a.pym, ev[k]));
        st<T>(H[k] + j, cmul(a.pym, h[k]));
      }
  }
  if (z == g.nz) {
    const long j = g.at(x, y, 0);
#pragma unroll
    for (int k = 0; k < 3; ++k)
      if (MASK & (1 << k)) {
        st<T>(Ec[k] + j, cmul(a.pzm, ev[k]));
        st<T>(H[k] + j, cmul(a.pzm, h[k]));
      }
  }
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
__device__ inline void incident(const SrcArgs& s, int ix, int iz, int it, cx<double>& ta, cx<double>& tb) {
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

// The two corrections of one column at one step, as tabulated for the
// persistent kernel.
struct __align__(32) TfsfVal {
  double er, ei, hr, hi;  // vE, vH
};

// The two corrections of column ix at step it: vE (added to or subtracted
// from E at iz_min) and vH (at iz_min-1 in variant 1, iz_min in variant 2).
// They depend on (ix, it) only: the incident field is y-independent.
__device__ __forceinline__ void tfsf_values(const SrcArgs& s, int it, int ix, cx<double>& vE, cx<double>& vH) {
  const int zm = s.iz_min;
  if (s.variant == 1) {
    cx<double> a0, b0, a1, b1;
    incident(s, ix, zm - 1, it, a0, b0);  // tfsf_data(:, ix, iy, iz_min-1)
    incident(s, ix, zm, it, a1, b1);      // tfsf_data(:, ix, iy, iz_min)
    vE = {dm(s.eps_in1, b0.re), dm(s.eps_in1, b0.im)};
    vH = {dm(s.dtcq2, a1.re), dm(s.dtcq2, a1.im)};
  } else if (s.variant == 2) {
    cx<double> ta, tb;
    incident(s, ix, zm, it, ta, tb);
    vE = {dq(tb.re, s.eps_src), dq(tb.im, s.eps_src)};
    vH = {dm(s.dtcq2, ta.re), dm(s.dtcq2, ta.im)};
  } else {
    vE = {0.0, 0.0};
    vH = {0.0, 0.0};
  }
}

// The corrections of column ix over the rows iy in [y0, y1]
// (code/tfsf.f90:76-153, :163-227).
template <typename T>
__device__ __forceinline__ void tfsf_apply(typename V2<T>::t* e, typename V2<T>::t* h, const Geo& g,
                                           const SrcArgs& s, int ix, int y0, int y1, cx<double> vE, cx<double> vH) {
  const int zm = s.iz_min;
  if (!bc_ok(ix >= 0 && ix <= s.nx + 1 && y0 >= 0 && y1 <= s.ny + 1 && zm >= 1 && zm <= g.nz, BC_TFSF,
             ((long)ix << 32) | (unsigned)y1))
    return;
  if (s.variant == 1) {
    if (s.i_pol == 2) {
      // E_x(iz_min) += eps_in(1)*tf5(iz_min-1): ix in [0,nx], iy in [0,ny+1]
      // H_y(iz_min-1) += dtcq2*tf1(iz_min):      ix in [0,nx], iy in [0,ny+1]
      for (int iy = y0; iy <= y1; ++iy) {
        if (ix <= s.nx && iy <= s.ny + 1) corr<T>(e + g.at(ix, iy, zm), vE, +1);
        if (ix <= s.nx && iy <= s.ny + 1) corr<T>(h + g.comp + g.at(ix, iy, zm - 1), vH, +1);
      }
    } else {
      // E_y(iz_min) -= eps_in(1)*tf4(iz_min-1): ix in [0,nx+1], iy in [0,ny]
      // H_x(iz_min-1) -= dtcq2*tf2(iz_min):      ix in [0,nx+1], iy in [0,ny]
      for (int iy = y0; iy <= y1; ++iy) {
        if (ix <= s.nx + 1 && iy <= s.ny) corr<T>(e + g.comp + g.at(ix, iy, zm), vE, -1);
        if (ix <= s.nx + 1 && iy <= s.ny) corr<T>(h + g.at(ix, iy, zm - 1), vH, -1);
      }
    }
  } else if (s.variant == 2) {
    // E_x(iz_min) += tf5(iz_min)/eps ; H_y(iz_min) += dtcq2*tf1(iz_min)
    for (int iy = y0; iy <= y1; ++iy) {
      corr<T>(e + g.at(ix, iy, zm), vE, +1);
      corr<T>(h + g.comp + g.at(ix, iy, zm), vH, +1);
    }
  }
}

// Incident field at ix and the corrections of the rows iy in [y0, y1].
template <typename T>
__device__ __forceinline__ void tfsf_column(typename V2<T>::t* e, typename V2<T>::t* h, const Geo& g,
                                            const SrcArgs& s, int it, int ix, int y0, int y1) {
  cx<double> vE, vH;
  tfsf_values(s, it, ix, vE, vH);
  tfsf_apply<T>(e, h, g, s, ix, y0, y1, vE, vH);
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
// Samples of one run handled by a block of 256 threads: GATHER_PER per
// thread, their loads issued before their stores.  Sample L of the run is
// location (u, v) = (L mod nu, L div nu); runs hold fewer than 2^31 samples.
constexpr int GATHER_PER = 4, GATHER_BLOCK = 256 * GATHER_PER;
// comp: elements of a field component, np: points of a ring slot (checked
// by the bounds-check build).
template <typename T>
__device__ __forceinline__ void gather_run(const Seg& sg, const typename V2<T>::t* __restrict__ src,
                                           typename V2<T>::t* __restrict__ slot, long comp, long np) {
  using V = typename V2<T>::t;
  const unsigned n = (unsigned)sg.nu * (unsigned)sg.nv, nu = (unsigned)sg.nu;
  const unsigned L0 = blockIdx.x * (unsigned)GATHER_BLOCK + threadIdx.x;
  V val[GATHER_PER];
#pragma unroll
  for (int j = 0; j < GATHER_PER; ++j) {
    const unsigned L = L0 + 256u * j;
    if (L < n) {
      const unsigned v = L / nu, u = L - v * nu;
      const long q = sg.src + (long)u * sg.su + (long)v * sg.sv;
      val[j] = bc_ok(q >= 0 && q < comp, BC_GATHER_SRC, q) ? src[q] : V{};
    }
  }
#pragma unroll
  for (int j = 0; j < GATHER_PER; ++j) {
    const unsigned L = L0 + 256u * j;
    if (L < n && bc_ok(sg.p0 + L < np, BC_GATHER_DST, sg.p0 + L)) slot[sg.p0 + L] = val[j];
  }
}

// Poynting flux of one face, code/dataprocess.f90:246-277:
// J = sign * sum Re(a*conj(b) - c*conj(d)) * eps0*Q/(2 dt).
struct FluxFace {
  long pa, pb, pc, pd;  // first sample index of the four components
  long n;               // locations on the face
  int sign, active;
};

}  // namespace iris
