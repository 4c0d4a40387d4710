// The fused E+H pass of one tile column (FP32), shared by the single-engine
// launch (iris_engine.cu) and the batched form (iris_batch.cu).  Not part of
// the public ABI.
#pragma once
#include <cuda_runtime.h>

#include "iris_device.cuh"

namespace iris {

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
//
// Loads: a thread's own E and H of the next plane go to registers one plane
// ahead.  What it reads after the barrier from outside the tile (the H
// neighbours at x-1 for lane 0 and at y-1 for warp 0, and the ghosts the
// image threads read) and the eps_inv of structure planes would otherwise be
// dependent loads right after the barrier, which every warp waits for; they
// are copied into shared memory by cp.async one plane ahead instead, into
// slots only the issuing thread reads.
//
// A step is two launches over z chunks (chunks are independent: each reads
// the old state of its planes and the plane below and above it): the planes
// pmlzi+1 .. pmlzf-2 by the kernel compiled without UPML code (UPML =
// false), and the two slabs, each with the one plane next to it, by the
// kernel with it, the two on separate streams so that they run
// concurrently (they write disjoint planes).  The interior range stops at pmlzf-2 because a chunk also
// computes E' one plane past its end (its last H' needs it), and that plane
// must not lie in a slab.

constexpr int FZ_X = 32, FZ_Y = 16, FZ_OX = FZ_X - 1, FZ_OY = FZ_Y - 1;

struct FusedArgs {
  FieldArgs<float> f;  // the old state: f.e, f.h, f.pml_d (D old), f.pml_b (B, in place)
  float2* e_new;
  float2* h_new;
  float2* d_new[2];
  // z chunks: blockIdx.z < nc0 covers planes za0 + zc0 * blockIdx.z on (at
  // most zc0, up to zb0), the rest the same over za1..zb1
  int za0, zb0, zc0, nc0, za1, zb1, zc1;
};

// Dynamic shared memory of the slab kernel (UPML = true): this thread's old
// D of the plane and B of the plane below, and the two planes' coefficient
// rows, copied one plane ahead like the halo.
struct FusedUpml {
  cx<float> d[2][FZ_Y][FZ_X][3];
  cx<float> b[2][FZ_Y][FZ_X][3];
  // [plane mod 3][E row of the plane, H row of the plane below]: read by
  // every thread, so three slots: the refill for plane z+1, issued before
  // plane z's barrier, must not land in the slot that slower warps may
  // still be reading for plane z-1
  float cf[3][2][NCOEF];
};
constexpr size_t FZ_UPML_SMEM = sizeof(FusedUpml);

__device__ __forceinline__ cx<float> shfl_cx(cx<float> v, int d, bool up) {
  cx<float> r;
  r.re = up ? __shfl_up_sync(0xffffffffu, v.re, d) : __shfl_down_sync(0xffffffffu, v.re, d);
  r.im = up ? __shfl_up_sync(0xffffffffu, v.im, d) : __shfl_down_sync(0xffffffffu, v.im, d);
  return r;
}

__device__ __forceinline__ void cpa8(void* dst, const void* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cpa4(void* dst, const void* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cpa_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N> __device__ __forceinline__ void cpa_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

// Static shared memory of one tile column of the fused pass.
struct FusedSmem {
  // per row and plane parity: H(z) components 1, 3 and E'(z-1) components 1, 3
  float2 xr[2][FZ_Y][4][FZ_X];
  // H neighbours outside the tile, copied one plane ahead (plane parity):
  // x-1 components 1, 2 for lane 0 [0] and the x-image lane [1]; y-1
  // components 0, 2 for warp 0 [0] and the y-image warp [1]
  float2 xh[2][FZ_Y][2][2];
  float2 yh[2][2][2][FZ_X];
  float epsh[2][FZ_Y][FZ_X];  // eps_inv of a structure plane (real material)
};

// Planes z0..z1 of column tile (bx, by), called by every thread of the CTA;
// U is used by UPML = true only.  IT: the integer type of the element offsets
// of the per-plane loads and stores (int when every offset of the three field
// components fits, which saves the 64-bit index arithmetic of every access;
// long otherwise).
template <bool CEPS, bool UPML, typename IT = long>
__device__ __forceinline__ void fused_column(const FusedArgs& A, FusedSmem& S, FusedUpml& U, int bx, int by, int z0,
                                             int z1) {
  const FieldArgs<float>& a = A.f;
  const Geo& g = a.g;
  auto& xr = S.xr;
  auto& xh = S.xh;
  auto& yh = S.yh;
  auto& epsh = S.epsh;
  const int lane = threadIdx.x, w = threadIdx.y;
  const int x = 1 + bx * FZ_OX + lane, y = 1 + by * FZ_OY + w;
  if (!bc_ok(z0 >= 1 && z1 <= g.nz && z0 <= z1 + 1, BC_FUSED_CELL, ((long)z0 << 32) | (unsigned)z1)) return;
  const bool act = x <= g.nx + 1 && y <= g.ny + 1;
  const bool ximg = x == g.nx + 1, yimg = y == g.ny + 1;
  const int cxx = ximg ? 1 : x, cyy = yimg ? 1 : y;  // the cell whose E' this thread computes
  const bool own = lane < FZ_OX && w < FZ_OY && x <= g.nx && y <= g.ny;
  cx<float> ph = {1.f, 0.f};
  if (ximg) ph = cmul(ph, a.pxp);
  if (yimg) ph = cmul(ph, a.pyp);
  const float2* E = a.e;
  const float2* H = a.h;
  // element offsets: plane, row, component, and this thread's columns
  // (cxx, cyy) for what it reads and (x, y) for what it writes
  const IT pl = (IT)g.plane, pt = (IT)g.pitch, cp = (IT)g.comp;
  const IT oc = (IT)cyy * pt + (IT)(cxx + g.xo), ow = (IT)y * pt + (IT)(x + g.xo);
  auto ldc = [&](const float2* f, int k, int zz) { return ld<float>(f + ((IT)k * cp + (IT)zz * pl + oc)); };
  const bool xhalo = act && (lane == 0 || ximg), yhalo = act && (w == 0 || yimg);
  const int xs = lane == 0 ? 0 : 1, ys = w == 0 ? 0 : 1;
  // The copies of plane p in [z0, z1 + 1] (plane nz + 1 is the image of
  // plane 1) into the slots of parity p & 1: one commit group per plane.
  auto ahead = [&](int p) {
    if (p <= z1 + 1) {
      const int zp = p == g.nz + 1 ? 1 : p;
      if (!CEPS && act && zp >= a.hi && zp <= a.hf)
        cpa4(&epsh[p & 1][w][lane], a.eps_r + ((IT)(zp - a.hi) * pl + oc));
      if (xhalo) {
        const IT q = (IT)zp * pl + oc - 1;
        cpa8(&xh[p & 1][w][xs][0], H + (cp + q));
        cpa8(&xh[p & 1][w][xs][1], H + (2 * cp + q));
      }
      if (yhalo) {
        const IT q = (IT)zp * pl + oc - pt;
        cpa8(&yh[p & 1][ys][0][lane], H + q);
        cpa8(&yh[p & 1][ys][1][lane], H + (2 * cp + q));
      }
      if (UPML) {
        // the old D of this thread's E' cell on plane zp, the B of its H'
        // cell on plane p-1, and both planes' coefficient rows (warps 0, 1)
        const int zb = p - 1;
        const bool pe = zp <= a.pmlzi || zp >= a.pmlzf, pb = zb >= z0 && (zb <= a.pmlzi || zb >= a.pmlzf);
        if (act && pe) {
          const int slab = zp <= a.pmlzi ? 0 : 1, zr = slab == 0 ? zp - 1 : zp - a.pmlzf;
          const long pi = ((long)zr * g.ny + (cyy - 1)) * (long)g.nx + (cxx - 1);
          if (bc_ok(pi >= 0 && pi < a.pcomp[slab], BC_FUSED_SLAB, pi))
#pragma unroll
            for (int k = 0; k < 3; ++k) cpa8(&U.d[p & 1][w][lane][k], a.pml_d[slab] + k * a.pcomp[slab] + pi);
        }
        if (own && pb) {
          const int slab = zb <= a.pmlzi ? 0 : 1, zr = slab == 0 ? zb - 1 : zb - a.pmlzf;
          const long pi = ((long)zr * g.ny + (y - 1)) * (long)g.nx + (x - 1);
          if (bc_ok(pi >= 0 && pi < a.pcomp[slab], BC_FUSED_SLAB, pi))
#pragma unroll
            for (int k = 0; k < 3; ++k) cpa8(&U.b[p & 1][w][lane][k], a.pml_b[slab] + k * a.pcomp[slab] + pi);
        }
        if (w < 2 && lane < NCOEF && (w == 0 ? pe : pb)) {
          const int zz = w == 0 ? zp : zb;
          const int row = zz <= a.pmlzi ? zz - 1 : a.pmlzi + zz - a.pmlzf;
          cpa4(&U.cf[p % 3][w][lane], a.coef + NCOEF * row + lane);
        }
      }
    }
    cpa_commit();
  };
  ahead(z0);
  const cx<float> zero = {0.f, 0.f};
  // Carried from plane z-1 in this thread's own slots of the exchange rows
  // (written there for the neighbours anyway): components 1, 3 of H(z-1) in
  // rows of parity (z-1)&1 and of E'(z-1) in rows of parity z&1 (stored at
  // the end of the previous plane); component 2 of both in registers.
  cx<float> ep1 = zero, hp1 = act ? ldc(H, 1, z0 - 1) : zero;
  {
    const cx<float> h0 = act ? ldc(H, 0, z0 - 1) : zero, h2 = act ? ldc(H, 2, z0 - 1) : zero;
    xr[(z0 - 1) & 1][w][0][lane] = make_float2(h0.re, h0.im);
    xr[(z0 - 1) & 1][w][1][lane] = make_float2(h2.re, h2.im);
    xr[z0 & 1][w][2][lane] = make_float2(0.f, 0.f);
    xr[z0 & 1][w][3][lane] = make_float2(0.f, 0.f);
  }
  cx<float> en[3], hn_[3];  // E and H of the next plane, loaded one plane ahead
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    en[k] = act ? ldc(E, k, z0) : zero;
    hn_[k] = act ? ldc(H, k, z0) : zero;
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
        en[k] = ldc(E, k, zn);
        hn_[k] = ldc(H, k, zn);
      }
    }
    ahead(z + 1);
    if (zimg && act) {
      hzm0 = ldc(H, 0, 0);
      hzm1 = ldc(H, 1, 0);
    } else {
      hzm0 = hp[0];
      hzm1 = hp[1];
    }
    xr[buf][w][0][lane] = make_float2(h[0].re, h[0].im);
    xr[buf][w][1][lane] = make_float2(h[2].re, h[2].im);
    cx<float> hx1 = shfl_cx(h[1], 1, true), hx2 = shfl_cx(h[2], 1, true);
    const cx<float> ex1 = shfl_cx(ep[1], 1, false), ex2 = shfl_cx(ep[2], 1, false);
    // this thread's copies of plane z have landed (those of z + 1 may not);
    // the barrier then shows the coefficient rows to every thread
    cpa_wait<1>();
    __syncthreads();
    cx<float> enew[3];
    if (act) {
      if (xhalo) {
        const float2 u = xh[z & 1][w][xs][0], v = xh[z & 1][w][xs][1];
        hx1 = {u.x, u.y};
        hx2 = {v.x, v.y};
      }
      cx<float> hy0, hy2;
      if (yhalo) {
        const float2 u = yh[z & 1][ys][0][lane], v = yh[z & 1][ys][1][lane];
        hy0 = {u.x, u.y};
        hy2 = {v.x, v.y};
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
      e_apply<float, CEPS, 7, !CEPS, UPML>(a, (own && z <= z1) ? A.d_new : nullptr, cxx, cyy, cz, c, enew,
                                           CEPS ? 0.f : epsh[z & 1][w][lane], UPML ? U.d[z & 1][w][lane] : nullptr,
                                           UPML ? U.cf[z % 3][0] : nullptr);
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
        h_update<float, UPML>(a, x, y, z - 1, ep, xp, yp, zp, hn, UPML ? U.b[z & 1][w][lane] : nullptr,
                              UPML ? U.cf[z % 3][1] : nullptr);
        const IT i = (IT)(z - 1) * pl + ow;
#pragma unroll
        for (int k = 0; k < 3; ++k) st<float>(A.h_new + ((IT)k * cp + i), hn[k]);
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
        const IT i = (IT)z * pl + ow;
#pragma unroll
        for (int k = 0; k < 3; ++k) st<float>(A.e_new + ((IT)k * cp + i), enew[k]);
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


}  // namespace iris
