// GB300 (sm_103a) FDTD engine, adjoint (gradient) form.

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "iris_engine.h"

using namespace iris;

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

unsigned long long bc_take_adjoint() { return bc_take_module(); }

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
// The DFT values in FP64: FP64-mode accumulators, or FP32 mode's
// double-float pairs (re_hi, im_hi, re_lo, im_lo).
__device__ __forceinline__ double2 adj_acc(const void* fd, long i, bool df) {
  if (!df) return ((const double2*)fd)[i];
  const float4 a = ((const float4*)fd)[i];
  return make_double2((double)a.x + (double)a.z, (double)a.y + (double)a.w);
}

template <typename T>
__global__ void __launch_bounds__(256) k_adj_source(typename V2<T>::t* __restrict__ ae, typename V2<T>::t* __restrict__ ah,
                                                    Geo g, const void* __restrict__ fd, long P, AdjFace f,
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
  const bool df = sizeof(T) == 4;  // FP32 mode: double-float accumulators
  for (int iw = 0; iw < nof; ++iw) {
    const long row = (long)iw * P;
    const double2 xe = adj_acc(fd, row + f.b[0] + L, df), ye = adj_acc(fd, row + f.b[1] + L, df);
    const double2 xh = adj_acc(fd, row + f.b[3] + L, df), yh = adj_acc(fd, row + f.b[4] + L, df);
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
  CK(cudaMemsetAsync(F->fd, 0, (size_t)F->P * F->p.nof * 16, F->st));
  F->fd_zero = false;
  F->nslot = 0;
  CK(cudaEventRecord(J->ev[0], F->st));
  for (int it = 1; it <= nsteps; ++it) {
    const int seg = (it - 1) / J->K;
    if ((it - 1) % J->K == 0) {
      rc = ckpt_io(J, seg, true);
      if (rc) return rc;
    }
    if (seg == S - 1) adj_record<T>(J, it - 1 - seg * J->K);
    one_step(F, it, true);
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
        one_step(F, it, false);
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
  // the forward engine steps as the parameters ask (FP32: the fused pass by
  // default); the adjoint state is a member engine that only holds fields
  iris_params q = p;
  for (int i = 0; i < 6; ++i) q.box2[i] = q.box1[i];
  int rc = create_engine(&q, fw, false, true, &J->F);
  if (rc) return bail(rc);
  q.stencil = IRIS_STENCIL_SPLIT;
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
  iris::NvtxRange nvtx_("iris_adjoint_forward");
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
  iris::NvtxRange nvtx_("iris_adjoint_backward");
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
