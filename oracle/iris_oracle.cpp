// TEST INFRASTRUCTURE ONLY — the parity oracle for the GB300 FDTD engine.
//
// A CPU, FP64, single-address-space restatement of the IrisFDTD-Academic hot
// path (Fortran, code/*.f90).  Only tests/, __graft_entry__.smoke() and the
// cpu_baseline leg of bench.py load this library, and only as the checker or
// the timed CPU baseline; the product never links or calls it.
//
// Layout and arithmetic follow the Fortran on purpose, so that every
// floating-point operation happens in the same order as the reference:
//   * fields are complex(8) arrays (3, 0:nx+1, 0:ny+1, 0:nz+1), component
//     fastest (code/main.f90:166-167, code/driver.f90:301-302), double
//     buffered with a pointer swap each step (code/driver.f90:358-384);
//   * complex products are the plain (ac-bd, ad+bc) form and the library is
//     built with -ffp-contract=off (no FMA), as a default x86 Fortran build;
//   * every loop range is the reference's, ghosts included.
// The one deliberate change: scattering_fourier evaluates cdexp(ci*w*it) once
// per (frequency, step) instead of once per sample point
// (code/dataprocess.f90:144); the value is identical because it does not
// depend on the point.
//
// Parity of this restatement is pinned in tests/test_oracle_pins.py against
// the reference's own numbers (dt and step count of example_1 quoted in
// irisfdtd_movie.py:25) and the analytic film spectrum the reference writes
// (code/common.f90:104-131); tests/test_oracle_properties.py checks its Bloch
// wrap (periodic supercells) and its linearity in the source.  The reference
// itself cannot be compiled here (no Fortran compiler), so bit-level pinning
// against a reference run is not possible.

#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

struct C {
  double re, im;
};
inline C cadd(C a, C b) { return {a.re + b.re, a.im + b.im}; }
inline C csub(C a, C b) { return {a.re - b.re, a.im - b.im}; }
inline C cmul(C a, C b) { return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
inline C rmul(double r, C a) { return {r * a.re, r * a.im}; }
inline C cexp_i(double phi) { return {std::cos(phi), std::sin(phi)}; }  // exp((0,phi))
// Fortran cdexp of a general complex argument: exp(re)*(cos im, sin im)
inline C cexp_c(C z) {
  double m = std::exp(z.re);
  return {m * std::cos(z.im), m * std::sin(z.im)};
}
// Smith's complex division, as gfortran does it (used at set-up only).
inline C cdiv(C a, C b) {
  if (std::fabs(b.re) >= std::fabs(b.im)) {
    double r = b.im / b.re, den = b.re + b.im * r;
    return {(a.re + a.im * r) / den, (a.im - a.re * r) / den};
  } else {
    double r = b.re / b.im, den = b.re * r + b.im;
    return {(a.re * r + a.im) / den, (a.im * r - a.re) / den};
  }
}

}  // namespace

extern "C" {

// Run parameters after setparam() (code/files.f90:39-344), in a.u.
typedef struct orc_params {
  int nx, ny, nz;          // ixmax, iymax, izmax
  int pmlzi, pmlzf, npml;  // UPML slabs 1..pmlzi and pmlzf..nz, exponent nPML
  int hi, hf;              // structure z-range
  int i_pol;               // 1: E//y, 2: E//x
  int plane_wave;          // 1: tfsf_gauss, 0: tfsf_plane_wave
  int cosine;              // 1: real-valued source
  int iz_min, iz_max;      // TF/SF box planes (tfsf_zi, tfsf_zi+5)
  int nof;                 // number of DFT frequencies
  int to_fourier, sample_fourier;
  int box1[6];             // sxi sxf syi syf szi szf
  int box2[6];             // mxi mxf myi myf mzi mzf
  int system_model;        // never set by the reference: 0
  int texit;               // number of steps
  int no_downloads;        // output interval in steps, int(texit/no_downloads)
  double Q, dt, c0, pi, eps0, mu0, f_abohr;
  double eps1, eps3, eps_bbox_re, eps_bbox_im;
  double wzpml, pmlalfa;
  double epump, wlpump, gpump, zopump;  // tfsf_gauss(it,zopump,Epump,wlpump,Gpump)
  double eoxy, tincr, tdecay, gap;      // tfsf_plane_wave
  double ratio_angle;
  double akx_re, akx_im, aky_re, aky_im, akz_re, akz_im;
} orc_params;

struct orc_state {
  orc_params p;
  std::vector<double> fw;
  int nx, ny, nz;
  long sx, sy, sz;  // strides in complex elements of a field array
  std::vector<C> ebuf[2], hbuf[2];
  C *e_cur, *e_prev, *h_cur, *h_prev;
  // eps_inv(1,1,0:nx+1,0:ny+1,hi-1:hf+1)
  std::vector<C> eps_inv;
  // UPML: d/b (3,1:nx,1:ny,slab) for the two slabs, cur/prev
  std::vector<C> dbuf[2][2], bbuf[2][2];  // [slab][cur/prev-buffer]
  C *d_cur[2], *d_prev[2], *b_cur[2], *b_prev[2];
  std::vector<double> fpzmn, fmzmn, fpzmx, fmzmx;  // (3, n)
  int nbot, ntop;                                   // pmlzi, nz-pmlzf+1
  // tfsf_data(1:6, ix_min-1:ix_max+1, iy_min-1:iy_max+1, iz_min-1:iz_max+1)
  std::vector<C> tfsf;
  int tf_nx, tf_ny, tf_nz;
  // DFT: per box, three face pairs; pto(i,1:4) and fdata(i, iw)
  int nboxes;
  std::vector<int> pto[2][3];
  std::vector<C> fdata[2][3];
  long npts[2][3];
  int nthreads;
};

static inline long fidx(const orc_state* s, int c, int x, int y, int z) {
  return (long)(c - 1) + 3L * ((long)x + s->sx * (long)y + s->sy * (long)z);
}
static inline C& F(C* f, const orc_state* s, int c, int x, int y, int z) {
  return f[fidx(s, c, x, y, z)];
}
static inline long epsidx(const orc_state* s, int x, int y, int z) {
  return (long)x + (long)(s->nx + 2) * ((long)y + (long)(s->ny + 2) * (long)(z - (s->p.hi - 1)));
}
// pml(3,1:nx,1:ny,z0:z1) indexing, z relative to the slab start
static inline long pmlidx(const orc_state* s, int c, int x, int y, int zrel) {
  return (long)(c - 1) + 3L * ((long)(x - 1) + (long)s->nx * ((long)(y - 1) + (long)s->ny * (long)zrel));
}
static inline long tfidx(const orc_state* s, int c, int x, int y, int z) {
  // x in [-1, nx+2], y in [-1, ny+2], z in [iz_min-1, iz_max+1]
  return (long)(c - 1) + 6L * ((long)(x + 1) + (long)s->tf_nx * ((long)(y + 1) + (long)s->tf_ny * (long)(z - (s->p.iz_min - 1))));
}

// ---------------------------------------------------------------------------
// set_sz, code/boundary_II.f90:224-276.  Integer powers stay integer; the
// bottom and top slabs associate the product differently, as written there.
static void set_sz(orc_state* s) {
  const orc_params& p = s->p;
  int nb = p.pmlzi, nt = p.nz - p.pmlzf + 1;
  s->fpzmn.assign(3 * nb, 0.0);
  s->fmzmn.assign(3 * nb, 0.0);
  s->fpzmx.assign(3 * nt, 0.0);
  s->fmzmx.assign(3 * nt, 0.0);
  for (int i = 1; i <= nb; ++i) {
    long ip = 1;
    for (int k = 0; k < p.npml; ++k) ip *= (long)(p.pmlzi - i);
    double den = std::pow((double)(p.pmlzi - 1), p.npml);
    double sg3 = std::sqrt(p.eps1) * p.wzpml * ((double)ip / den);
    double k3 = 1.0 + std::sqrt(p.eps1) * p.pmlalfa * ((double)ip / den);
    for (int c = 0; c < 3; ++c) {
      double sg = (c == 2) ? sg3 : 0.0, k = (c == 2) ? k3 : 1.0;
      s->fpzmn[c + 3 * (i - 1)] = 2 * p.eps0 * p.eps1 * k + p.dt * sg;
      s->fmzmn[c + 3 * (i - 1)] = 2 * p.eps0 * p.eps1 * k - p.dt * sg;
    }
  }
  for (int i = p.pmlzf; i <= p.nz; ++i) {
    long ip = 1;
    for (int k = 0; k < p.npml; ++k) ip *= (long)(i - p.pmlzf);
    double den = std::pow((double)(p.nz - p.pmlzf), p.npml);
    double sg3 = std::sqrt(p.eps3) * p.wzpml * (double)ip / den;
    double k3 = 1.0 + std::sqrt(p.eps3) * p.pmlalfa * (double)ip / den;
    for (int c = 0; c < 3; ++c) {
      double sg = (c == 2) ? sg3 : 0.0, k = (c == 2) ? k3 : 1.0;
      s->fpzmx[c + 3 * (i - p.pmlzf)] = 2 * p.eps0 * p.eps3 * k + p.dt * sg;
      s->fmzmx[c + 3 * (i - p.pmlzf)] = 2 * p.eps0 * p.eps3 * k - p.dt * sg;
    }
  }
}

// init_store_pts_fourier, code/dataprocess.f90:793-903 (pto stored as 4 ints per point)
static void init_store_pts(orc_state* s, int nb) {
  const int* b = nb == 0 ? s->p.box1 : s->p.box2;
  int bxi = b[0], bxf = b[1], byi = b[2], byf = b[3], bzi = b[4], bzf = b[5];
  long np1 = 2L * 6 * (byf + 1 - byi) * (bzf + 1 - bzi);
  long np2 = 2L * 6 * (bxf + 1 - bxi) * (bzf + 1 - bzi);
  long np3 = 2L * 6 * (bxf + 1 - bxi) * (byf + 1 - byi);
  s->npts[nb][0] = np1;
  s->npts[nb][1] = np2;
  s->npts[nb][2] = np3;
  for (int j = 0; j < 3; ++j) {
    long n = s->npts[nb][j];
    bool alloc = (j == 0) ? (s->nx != 1) : (j == 1) ? (s->ny != 1) : true;
    if (!alloc) n = 1;
    s->pto[nb][j].assign(4 * n, 1);
    s->fdata[nb][j].assign(n * (long)s->p.nof, C{0.0, 0.0});
  }
  if (s->nx != 1) {
    int* pt = s->pto[nb][0].data();
    long half = 6L * (byf + 1 - byi) * (bzf + 1 - bzi);
    for (int side = 0; side < 2; ++side)
      for (int iy = 1; iy <= byf + 1 - byi; ++iy)
        for (int iz = 1; iz <= bzf + 1 - bzi; ++iz)
          for (int ip = 1; ip <= 6; ++ip) {
            long i = side * half + ip + 6L * (iy - 1 + (long)(byf + 1 - byi) * (iz - 1));
            int* q = pt + 4 * (i - 1);
            q[0] = ip; q[1] = side ? bxf : bxi; q[2] = iy + (byi - 1); q[3] = iz + (bzi - 1);
          }
  }
  if (s->ny != 1) {
    int* pt = s->pto[nb][1].data();
    long half = 6L * (bxf + 1 - bxi) * (bzf + 1 - bzi);
    for (int side = 0; side < 2; ++side)
      for (int ix = 1; ix <= bxf + 1 - bxi; ++ix)
        for (int iz = 1; iz <= bzf + 1 - bzi; ++iz)
          for (int ip = 1; ip <= 6; ++ip) {
            long i = side * half + ip + 6L * (ix - 1 + (long)(bxf + 1 - bxi) * (iz - 1));
            int* q = pt + 4 * (i - 1);
            q[0] = ip; q[1] = ix + (bxi - 1); q[2] = side ? byf : byi; q[3] = iz + (bzi - 1);
          }
  }
  {
    int* pt = s->pto[nb][2].data();
    long half = 6L * (bxf + 1 - bxi) * (byf + 1 - byi);
    for (int side = 0; side < 2; ++side)
      for (int ix = 1; ix <= bxf + 1 - bxi; ++ix)
        for (int iy = 1; iy <= byf + 1 - byi; ++iy)
          for (int ip = 1; ip <= 6; ++ip) {
            long i = side * half + ip + 6L * (ix - 1 + (long)(bxf + 1 - bxi) * (iy - 1));
            int* q = pt + 4 * (i - 1);
            q[0] = ip; q[1] = ix + (bxi - 1); q[2] = iy + (byi - 1); q[3] = side ? bzf : bzi;
          }
  }
}

static bool single_box(const orc_params& p) {
  for (int i = 0; i < 6; ++i)
    if (p.box1[i] != p.box2[i]) return false;
  return true;
}

int orc_create(const orc_params* pin, const double* fw, orc_state** out) {
  orc_state* s = new orc_state();
  s->p = *pin;
  const orc_params& p = s->p;
  s->nx = p.nx; s->ny = p.ny; s->nz = p.nz;
  s->sx = p.nx + 2;
  s->sy = (long)(p.nx + 2) * (p.ny + 2);
  s->sz = s->sy * (p.nz + 2);
  s->fw.assign(fw, fw + p.nof);
  long n = 3 * s->sz;
  for (int i = 0; i < 2; ++i) {
    s->ebuf[i].assign(n, C{0, 0});
    s->hbuf[i].assign(n, C{0, 0});
  }
  // main.f90 allocates e,h (the driver's initial e_cur,h_cur); driver allocates e_prev,h_prev
  s->e_cur = s->ebuf[0].data(); s->e_prev = s->ebuf[1].data();
  s->h_cur = s->hbuf[0].data(); s->h_prev = s->hbuf[1].data();
  // set_emconstants, code/mesh.f90:102-106
  long ne = (long)(p.nx + 2) * (p.ny + 2) * (p.hf - p.hi + 3);
  C one{1.0, 0.0};
  C inv_bbox = cdiv(one, C{p.eps_bbox_re, p.eps_bbox_im});
  s->eps_inv.assign(ne, inv_bbox);
  for (int y = 0; y <= p.ny + 1; ++y)
    for (int x = 0; x <= p.nx + 1; ++x) {
      s->eps_inv[epsidx(s, x, y, p.hi - 1)] = C{1.0 / p.eps1, 0.0};
      s->eps_inv[epsidx(s, x, y, p.hf + 1)] = C{1.0 / p.eps3, 0.0};
    }
  // UPML slabs, code/driver.f90:177-198
  s->nbot = p.pmlzi;
  s->ntop = p.nz - p.pmlzf + 1;
  for (int k = 0; k < 2; ++k) {
    long m = 3L * p.nx * p.ny * (k == 0 ? s->nbot : s->ntop);
    for (int q = 0; q < 2; ++q) {
      s->dbuf[k][q].assign(m, C{0, 0});
      s->bbuf[k][q].assign(m, C{0, 0});
    }
    s->d_cur[k] = s->dbuf[k][0].data(); s->d_prev[k] = s->dbuf[k][1].data();
    s->b_cur[k] = s->bbuf[k][0].data(); s->b_prev[k] = s->bbuf[k][1].data();
  }
  set_sz(s);
  // DFT sample tables, code/driver.f90:205-286
  init_store_pts(s, 0);
  s->nboxes = 1;
  if (!single_box(p)) {
    init_store_pts(s, 1);
    s->nboxes = 2;
  }
  // TF/SF scratch, code/driver.f90:314-326: ix in [ix_min-1, ix_max+1] = [-1, nx+2]
  s->tf_nx = p.nx + 4;
  s->tf_ny = p.ny + 4;
  s->tf_nz = (p.iz_max + 1) - (p.iz_min - 1) + 1;
  s->tfsf.assign(6L * s->tf_nx * s->tf_ny * s->tf_nz, C{0, 0});
  s->nthreads = 1;
  *out = s;
  return 0;
}

void orc_destroy(orc_state* s) { delete s; }

void orc_set_threads(orc_state* s, int n) { s->nthreads = n < 1 ? 1 : n; }

// eps_inv values over (0:nx+1, 0:ny+1, hi-1:hf+1), x fastest, split re/im.
int orc_set_eps_inv(orc_state* s, const double* re, const double* im) {
  long ne = (long)s->eps_inv.size();
  for (long i = 0; i < ne; ++i) s->eps_inv[i] = C{re[i], im ? im[i] : 0.0};
  return 0;
}

// slit(), code/mesh.f90:57-69 (aix:afx air over hi:hf, all y)
void orc_slit(orc_state* s, int aix, int afx) {
  for (int z = s->p.hi; z <= s->p.hf; ++z)
    for (int y = 0; y <= s->ny + 1; ++y)
      for (int x = aix; x <= afx; ++x) s->eps_inv[epsidx(s, x, y, z)] = C{1.0, 0.0};
}

// ---------------------------------------------------------------------------
// e_fdtd, code/fdtd.f90:57-153
static inline void curl_h(const orc_state* s, const C* h, int x, int y, int z, C* c) {
  c[0] = cadd(csub(csub(F((C*)h, s, 3, x, y, z), F((C*)h, s, 3, x, y - 1, z)), F((C*)h, s, 2, x, y, z)), F((C*)h, s, 2, x, y, z - 1));
  c[1] = cadd(csub(csub(F((C*)h, s, 1, x, y, z), F((C*)h, s, 1, x, y, z - 1)), F((C*)h, s, 3, x, y, z)), F((C*)h, s, 3, x - 1, y, z));
  c[2] = cadd(csub(csub(F((C*)h, s, 2, x, y, z), F((C*)h, s, 2, x - 1, y, z)), F((C*)h, s, 1, x, y, z)), F((C*)h, s, 1, x, y - 1, z));
}
static inline void curl_e(const orc_state* s, const C* e, int x, int y, int z, C* c) {
  c[0] = cadd(csub(csub(F((C*)e, s, 3, x, y + 1, z), F((C*)e, s, 3, x, y, z)), F((C*)e, s, 2, x, y, z + 1)), F((C*)e, s, 2, x, y, z));
  c[1] = cadd(csub(csub(F((C*)e, s, 1, x, y, z + 1), F((C*)e, s, 1, x, y, z)), F((C*)e, s, 3, x + 1, y, z)), F((C*)e, s, 3, x, y, z));
  c[2] = cadd(csub(csub(F((C*)e, s, 2, x + 1, y, z), F((C*)e, s, 2, x, y, z)), F((C*)e, s, 1, x, y + 1, z)), F((C*)e, s, 1, x, y, z));
}

static void e_fdtd(orc_state* s) {
  const orc_params& p = s->p;
  double m1 = 1.0 / p.eps1, m3 = 1.0 / p.eps3;  // epsa_inv diagonals, code/mesh.f90:94-99
  auto region = [&](int z0, int z1, double m) {
#pragma omp parallel for num_threads(s->nthreads) schedule(static)
    for (int z = z0; z <= z1; ++z)
      for (int y = 1; y <= s->ny; ++y)
        for (int x = 1; x <= s->nx; ++x) {
          C c[3];
          curl_h(s, s->h_prev, x, y, z, c);
          // e = e_prev + m_i1*c1 + m_i2*c2 + m_i3*c3 with an exactly diagonal tensor
          for (int i = 0; i < 3; ++i) {
            C v = F(s->e_prev, s, i + 1, x, y, z);
            for (int j = 0; j < 3; ++j) v = cadd(v, rmul(i == j ? m : 0.0, c[j]));
            F(s->e_cur, s, i + 1, x, y, z) = v;
          }
        }
  };
  region(1 + p.pmlzi, p.hi - 1, m1);
#pragma omp parallel for num_threads(s->nthreads) schedule(static)
  for (int z = p.hi; z <= p.hf; ++z)
    for (int y = 1; y <= s->ny; ++y)
      for (int x = 1; x <= s->nx; ++x) {
        C c[3];
        curl_h(s, s->h_prev, x, y, z, c);
        C ei = s->eps_inv[epsidx(s, x, y, z)];
        for (int i = 0; i < 3; ++i)
          F(s->e_cur, s, i + 1, x, y, z) = cadd(F(s->e_prev, s, i + 1, x, y, z), cmul(ei, c[i]));
      }
  region(p.hf + 1, p.pmlzf - 1, m3);
}

// h_fdtd, code/fdtd.f90:157-248 (mu_inv_bbox = 1)
static void h_fdtd(orc_state* s, double dtcq2) {
  const orc_params& p = s->p;
  int zmx_eff = (p.pmlzf < p.hf) ? p.hf : p.pmlzf - 1;
  auto region = [&](int z0, int z1, double coef) {
#pragma omp parallel for num_threads(s->nthreads) schedule(static)
    for (int z = z0; z <= z1; ++z)
      for (int y = 1; y <= s->ny; ++y)
        for (int x = 1; x <= s->nx; ++x) {
          C c[3];
          curl_e(s, s->e_cur, x, y, z, c);
          for (int i = 0; i < 3; ++i)
            F(s->h_cur, s, i + 1, x, y, z) = csub(F(s->h_prev, s, i + 1, x, y, z), rmul(coef, c[i]));
        }
  };
  region(p.pmlzi, p.hi - 1, dtcq2);
  region(p.hi, p.hf, dtcq2 * 1.0);
  region(p.hf + 1, zmx_eff, dtcq2);
}

// UPML_Array_e, code/boundary_II.f90:60-138
static void upml_e(orc_state* s) {
  const orc_params& p = s->p;
  for (int slab = 0; slab < 2; ++slab) {
    int z0 = slab == 0 ? 1 : p.pmlzf, z1 = slab == 0 ? p.pmlzi : p.nz;
    const double* fp = slab == 0 ? s->fpzmn.data() : s->fpzmx.data();
    const double* fm = slab == 0 ? s->fmzmn.data() : s->fmzmx.data();
    double epsb = slab == 0 ? p.eps1 : p.eps3;
    C* dc = s->d_cur[slab];
    C* dp = s->d_prev[slab];
#pragma omp parallel for num_threads(s->nthreads) schedule(static)
    for (int z = z0; z <= z1; ++z) {
      int zr = z - z0;
      const double* fpz = fp + 3 * zr;
      const double* fmz = fm + 3 * zr;
      for (int y = 1; y <= s->ny; ++y)
        for (int x = 1; x <= s->nx; ++x) {
          C c[3];
          curl_h(s, s->h_prev, x, y, z, c);
          for (int i = 0; i < 3; ++i) c[i] = rmul(p.eps0 * p.eps0, c[i]);
          // component -> profile permutation, code/boundary_II.f90:86-99
          const int pd[3] = {1, 2, 0};  // D_i uses profile pd[i] for its own decay
          const int pe[3] = {2, 0, 1};  // E_i decays with profile pe[i]
          C dn[3], dold[3];
          for (int i = 0; i < 3; ++i) {
            dold[i] = dp[pmlidx(s, i + 1, x, y, zr)];
            dn[i] = cadd(rmul(fmz[pd[i]] / fpz[pd[i]], dold[i]), rmul((2 * epsb) / fpz[pd[i]], c[i]));
            dc[pmlidx(s, i + 1, x, y, zr)] = dn[i];
          }
          for (int i = 0; i < 3; ++i) {
            C v = rmul(fmz[pe[i]] / fpz[pe[i]], F(s->e_prev, s, i + 1, x, y, z));
            C w = csub(rmul(fpz[i], dn[i]), rmul(fmz[i], dold[i]));
            F(s->e_cur, s, i + 1, x, y, z) = cadd(v, rmul(1 / (p.eps0 * epsb * fpz[pe[i]]), w));
          }
        }
    }
  }
}

// UPML_Array_h, code/boundary_II.f90:142-220
static void upml_h(orc_state* s) {
  const orc_params& p = s->p;
  double dtq2 = (p.dt / p.Q) * (p.dt / p.Q);
  for (int slab = 0; slab < 2; ++slab) {
    int z0 = slab == 0 ? 1 : p.pmlzf, z1 = slab == 0 ? p.pmlzi : p.nz;
    const double* fp = slab == 0 ? s->fpzmn.data() : s->fpzmx.data();
    const double* fm = slab == 0 ? s->fmzmn.data() : s->fmzmx.data();
    double epsb = slab == 0 ? p.eps1 : p.eps3;
    C* bc = s->b_cur[slab];
    C* bp = s->b_prev[slab];
#pragma omp parallel for num_threads(s->nthreads) schedule(static)
    for (int z = z0; z <= z1; ++z) {
      int zr = z - z0;
      const double* fpz = fp + 3 * zr;
      const double* fmz = fm + 3 * zr;
      for (int y = 1; y <= s->ny; ++y)
        for (int x = 1; x <= s->nx; ++x) {
          C c[3];
          curl_e(s, s->e_cur, x, y, z, c);
          const int pd[3] = {1, 2, 0};
          const int pe[3] = {2, 0, 1};
          C bn[3], bold[3];
          for (int i = 0; i < 3; ++i) {
            bold[i] = bp[pmlidx(s, i + 1, x, y, zr)];
            bn[i] = csub(rmul(fmz[pd[i]] / fpz[pd[i]], bold[i]), rmul(((2 * epsb) / fpz[pd[i]]) * dtq2, c[i]));
            bc[pmlidx(s, i + 1, x, y, zr)] = bn[i];
          }
          for (int i = 0; i < 3; ++i) {
            C v = rmul(fmz[pe[i]] / fpz[pe[i]], F(s->h_prev, s, i + 1, x, y, z));
            C w = csub(rmul(fpz[i], bn[i]), rmul(fmz[i], bold[i]));
            F(s->h_cur, s, i + 1, x, y, z) = cadd(v, rmul(1 / (p.mu0 * fpz[pe[i]]), w));
          }
        }
    }
  }
}

// bc_{x,y,z}max_bloch / bc_{x,y,z}min_bloch, code/boundary.f90:163-348.
// ak are complex module variables; the reference never assigns them (0).
static C phase(double re, double im, int sgn) {
  // cdexp(sgn*ci*ak): ci*ak = (-im, re)
  C arg{-(double)sgn * im, (double)sgn * re};
  return cexp_c(arg);
}
static void bloch_max(orc_state* s) {
  const orc_params& p = s->p;
  C fx = phase(p.akx_re, p.akx_im, +1), fy = phase(p.aky_re, p.aky_im, +1), fz = phase(p.akz_re, p.akz_im, +1);
  for (int y = 1; y <= s->ny; ++y)
    for (int z = 1; z <= s->nz; ++z)
      for (int i = 1; i <= 3; ++i) {
        F(s->e_cur, s, i, s->nx + 1, y, z) = cmul(fx, F(s->e_cur, s, i, 1, y, z));
        F(s->h_cur, s, i, s->nx + 1, y, z) = cmul(fx, F(s->h_cur, s, i, 1, y, z));
      }
  for (int x = 1; x <= s->nx; ++x)
    for (int z = 1; z <= s->nz; ++z)
      for (int i = 1; i <= 3; ++i) {
        F(s->e_cur, s, i, x, s->ny + 1, z) = cmul(fy, F(s->e_cur, s, i, x, 1, z));
        F(s->h_cur, s, i, x, s->ny + 1, z) = cmul(fy, F(s->h_cur, s, i, x, 1, z));
      }
  for (int x = 1; x <= s->nx; ++x)
    for (int y = 1; y <= s->ny; ++y)
      for (int i = 1; i <= 3; ++i) {
        F(s->e_cur, s, i, x, y, s->nz + 1) = cmul(fz, F(s->e_cur, s, i, x, y, 1));
        F(s->h_cur, s, i, x, y, s->nz + 1) = cmul(fz, F(s->h_cur, s, i, x, y, 1));
      }
}
static void bloch_min(orc_state* s) {
  const orc_params& p = s->p;
  C fx = phase(p.akx_re, p.akx_im, -1), fy = phase(p.aky_re, p.aky_im, -1), fz = phase(p.akz_re, p.akz_im, -1);
  for (int y = 1; y <= s->ny; ++y)
    for (int z = 1; z <= s->nz; ++z)
      for (int i = 1; i <= 3; ++i) {
        F(s->e_cur, s, i, 0, y, z) = cmul(fx, F(s->e_cur, s, i, s->nx, y, z));
        F(s->h_cur, s, i, 0, y, z) = cmul(fx, F(s->h_cur, s, i, s->nx, y, z));
      }
  for (int x = 1; x <= s->nx; ++x)
    for (int z = 1; z <= s->nz; ++z)
      for (int i = 1; i <= 3; ++i) {
        F(s->e_cur, s, i, x, 0, z) = cmul(fy, F(s->e_cur, s, i, x, s->ny, z));
        F(s->h_cur, s, i, x, 0, z) = cmul(fy, F(s->h_cur, s, i, x, s->ny, z));
      }
  for (int x = 1; x <= s->nx; ++x)
    for (int y = 1; y <= s->ny; ++y)
      for (int i = 1; i <= 3; ++i) {
        F(s->e_cur, s, i, x, y, 0) = cmul(fz, F(s->e_cur, s, i, x, y, s->nz));
        F(s->h_cur, s, i, x, y, 0) = cmul(fz, F(s->h_cur, s, i, x, y, s->nz));
      }
}

// ---------------------------------------------------------------------------
// tfsf_gauss, code/tfsf.f90:231-355 (FTwindow = 0, so win = 1)
static void tfsf_gauss(orc_state* s, int it) {
  const orc_params& p = s->p;
  C* tf = s->tfsf.data();
  int ixo = p.pmlzi - 50, ito = 0;
  double izo = p.zopump;
  double Dk = p.gpump * p.Q;
  double ko = 2 * p.pi / (p.wlpump * p.f_abohr);
  double eps_src, sign_kz;
  if (p.iz_min > p.hi) { eps_src = p.eps3; sign_kz = -1.0; }
  else { eps_src = p.eps1; sign_kz = 1.0; }
  double DELTA = p.ratio_angle * p.pi / 2.0;
  double ux = std::cos(DELTA), uz = std::sin(DELTA);
  double win = 1.0;
  double amp = p.epump * p.Q;
  double hcoef = amp * (p.dt * p.c0 / p.Q);
#pragma omp parallel for num_threads(s->nthreads) schedule(static)
  for (int iy = -1; iy <= s->ny + 2; ++iy)
    for (int ix = -1; ix <= s->nx + 2; ++ix)
      for (int iz = p.iz_min - 1; iz <= p.iz_max + 1; ++iz) {
        double A = p.Q * (double)(ix - ixo) * ux + p.Q * ((double)iz - izo) * uz;
        double kzz = ko * (std::sqrt(eps_src) * sign_kz * A - p.c0 * p.dt * (double)(it - ito));
        double arg = (A - p.c0 * p.dt * (double)(it - ito) / std::sqrt(eps_src)) / Dk;
        double env = std::exp(-(arg * arg));
        C ekz = cexp_i(kzz);
        if (p.i_pol == 1) {
          C hx = rmul(uz, rmul(env, cmul(C{sign_kz, 0.0}, ekz)));
          hx = C{-hx.re, -hx.im};
          C hz = rmul(ux, rmul(env, cmul(C{1.0, 0.0}, ekz)));
          C ey = cmul(C{1.0, 0.0}, csub(rmul(ux, hz), rmul(uz * sign_kz, hx)));
          if (p.cosine == 1) {
            ey = C{(ey.re + ey.re) / 2.0, (ey.im - ey.im) / 2.0};
            hz = C{(hz.re + hz.re) / 2.0, (hz.im - hz.im) / 2.0};
            hx = C{(hx.re + hx.re) / 2.0, (hx.im - hx.im) / 2.0};
          }
          C& t4 = tf[tfidx(s, 4, ix, iy, iz)];
          C& t6 = tf[tfidx(s, 6, ix, iy, iz)];
          C& t2 = tf[tfidx(s, 2, ix, iy, iz)];
          t4 = cadd(t4, rmul(hcoef, hx));
          t6 = cadd(t6, rmul(hcoef, hz));
          t2 = cadd(t2, rmul(amp, ey));
        } else if (p.i_pol == 2) {
          C ex = rmul(uz, rmul(env, cmul(C{sign_kz, 0.0}, ekz)));
          C ez = rmul(ux, rmul(env, cmul(C{1.0, 0.0}, ekz)));
          ez = C{-ez.re, -ez.im};
          C hy = cmul(C{1.0, 0.0}, csub(rmul(uz * sign_kz, ex), rmul(ux, ez)));
          if (p.cosine == 1) {
            ex = C{(ex.re + ex.re) / 2.0, (ex.im - ex.im) / 2.0};
            ez = C{(ez.re + ez.re) / 2.0, (ez.im - ez.im) / 2.0};
            hy = C{(hy.re + hy.re) / 2.0, (hy.im - hy.im) / 2.0};
          }
          C& t1 = tf[tfidx(s, 1, ix, iy, iz)];
          C& t3 = tf[tfidx(s, 3, ix, iy, iz)];
          C& t5 = tf[tfidx(s, 5, ix, iy, iz)];
          t1 = cadd(t1, rmul(amp, ex));
          t3 = cadd(t3, rmul(amp, ez));
          t5 = cadd(t5, rmul(hcoef, hy));
        }
      }
  if (win != 1.0)
    for (auto& v : s->tfsf) v = rmul(win, v);
}

// tfsf_plane_wave, code/tfsf.f90:359-517 (CW with on/off ramps; GAP never set)
static void tfsf_plane_wave(orc_state* s, int it) {
  const orc_params& p = s->p;
  C* tf = s->tfsf.data();
  int ixo = p.pmlzi - 50, ito = 0;
  // izo is an INTEGER there: pmlzi-(3*GAP) truncated toward zero
  int izo = p.ratio_angle >= 0 ? (int)((double)p.pmlzi - 3.0 * p.gap) : (int)((double)p.nz + 3.0 * p.gap);
  double Dk = p.gap * p.Q;
  double ko = 2 * p.pi / (p.wlpump * p.f_abohr);
  double DELTA = p.ratio_angle * p.pi / 2.0;
  double ux = std::cos(DELTA), uz = std::sin(DELTA);
  double amp = p.eoxy * p.Q;
  double hcoef = amp * (p.dt * p.c0 / p.Q);
  double s1 = std::sqrt(p.eps1);
  for (auto& v : s->tfsf) v = C{0, 0};
#pragma omp parallel for num_threads(s->nthreads) schedule(static)
  for (int iy = -1; iy <= s->ny + 2; ++iy)
    for (int ix = -1; ix <= s->nx + 2; ++ix)
      for (int iz = p.iz_min - 1; iz <= p.iz_max + 1; ++iz) {
        double kzz = ko * ((p.Q * (double)(ix - ixo) * ux + p.Q * (double)(iz - izo) * uz) - p.c0 * p.dt * (double)(it - ito) / s1);
        double d = p.Q * std::fabs((double)(iz - izo));
        double g;
        if (p.c0 * p.dt * ((double)it - p.tincr) <= d)
          g = std::exp(-(d - p.c0 * p.dt * ((double)it - p.tincr)) / Dk);
        else if (p.c0 * p.dt * ((double)it - p.tdecay) >= d)
          g = std::exp((d - p.c0 * p.dt * ((double)it - p.tdecay)) / Dk);
        else
          g = 1.0;
        C ekz = cexp_i(kzz);
        if (p.i_pol == 1) {
          C hx = rmul(uz, rmul(g, cmul(C{1.0, 0.0}, ekz)));
          hx = C{-hx.re, -hx.im};
          C hz = rmul(ux, rmul(g, cmul(C{1.0, 0.0}, ekz)));
          C ey = rmul(s1, csub(rmul(ux, hz), rmul(uz, hx)));
          if (p.cosine == 1) {
            ey = C{(ey.re + ey.re) / 2.0, (ey.im - ey.im) / 2.0};
            hz = C{(hz.re + hz.re) / 2.0, (hz.im - hz.im) / 2.0};
            hx = C{(hx.re + hx.re) / 2.0, (hx.im - hx.im) / 2.0};
          }
          tf[tfidx(s, 4, ix, iy, iz)] = rmul(hcoef, hx);
          tf[tfidx(s, 6, ix, iy, iz)] = rmul(hcoef, hz);
          tf[tfidx(s, 2, ix, iy, iz)] = rmul(amp, ey);
        } else if (p.i_pol == 2) {
          C ex = rmul(uz, rmul(g, cmul(C{1.0, 0.0}, ekz)));
          C ez = rmul(ux, rmul(g, cmul(C{1.0, 0.0}, ekz)));
          ez = C{-ez.re, -ez.im};
          C hy = rmul(s1, csub(rmul(uz, ex), rmul(ux, ez)));
          if (p.cosine == 1) {
            ex = C{(ex.re + ex.re) / 2.0, (ex.im - ex.im) / 2.0};
            ez = C{(ez.re + ez.re) / 2.0, (ez.im - ez.im) / 2.0};
            hy = C{(hy.re + hy.re) / 2.0, (hy.im - hy.im) / 2.0};
          }
          tf[tfidx(s, 1, ix, iy, iz)] = rmul(amp, ex);
          tf[tfidx(s, 3, ix, iy, iz)] = rmul(amp, ez);
          tf[tfidx(s, 5, ix, iy, iz)] = rmul(hcoef, hy);
        }
      }
}

// tfsf_update_3DArray, code/tfsf.f90:76-153 (upper plane disabled at :122)
static void tfsf_update_3d(orc_state* s) {
  const orc_params& p = s->p;
  double dtcq2 = (p.dt * p.c0 / p.Q) * (p.dt * p.c0 / p.Q);
  double eps_in1 = 1.0 / p.eps1;
  const double mu_inv = 1.0;
  C* tf = s->tfsf.data();
  int ixmn = 0, ixmx = s->nx + 1, iymn = 0, iymx = s->ny + 1, zm = p.iz_min;
  for (int iy = iymn; iy <= iymx; ++iy)
    for (int ix = ixmn; ix <= ixmx - 1; ++ix)
      F(s->e_cur, s, 1, ix, iy, zm) = cadd(F(s->e_cur, s, 1, ix, iy, zm), rmul(eps_in1, tf[tfidx(s, 5, ix, iy, zm - 1)]));
  for (int iy = iymn; iy <= iymx - 1; ++iy)
    for (int ix = ixmn; ix <= ixmx; ++ix)
      F(s->e_cur, s, 2, ix, iy, zm) = csub(F(s->e_cur, s, 2, ix, iy, zm), rmul(eps_in1, tf[tfidx(s, 4, ix, iy, zm - 1)]));
  for (int iy = iymn; iy <= iymx - 1; ++iy)
    for (int ix = ixmn; ix <= ixmx; ++ix)
      F(s->h_cur, s, 1, ix, iy, zm - 1) = csub(F(s->h_cur, s, 1, ix, iy, zm - 1), rmul(dtcq2 * mu_inv, tf[tfidx(s, 2, ix, iy, zm)]));
  for (int iy = iymn; iy <= iymx; ++iy)
    for (int ix = ixmn; ix <= ixmx - 1; ++ix)
      F(s->h_cur, s, 2, ix, iy, zm - 1) = cadd(F(s->h_cur, s, 2, ix, iy, zm - 1), rmul(dtcq2 * mu_inv, tf[tfidx(s, 1, ix, iy, zm)]));
}

// tfsf_update_2DArray, code/tfsf.f90:163-227 (right boundary disabled at :204)
static void tfsf_update_2d(orc_state* s) {
  const orc_params& p = s->p;
  double dtcq2 = (p.dt * p.c0 / p.Q) * (p.dt * p.c0 / p.Q);
  const double mu_inv = 1.0;
  double eps_src = (p.iz_min > p.hi) ? p.eps3 : p.eps1;
  C* tf = s->tfsf.data();
  int zm = p.iz_min;
  for (int iy = 0; iy <= s->ny + 1; ++iy)
    for (int ix = 0; ix <= s->nx + 1; ++ix) {
      C t5 = tf[tfidx(s, 5, ix, iy, zm)], t4 = tf[tfidx(s, 4, ix, iy, zm - 1)];
      F(s->e_cur, s, 1, ix, iy, zm) = cadd(F(s->e_cur, s, 1, ix, iy, zm), C{t5.re / eps_src, t5.im / eps_src});
      F(s->e_cur, s, 2, ix, iy, zm) = csub(F(s->e_cur, s, 2, ix, iy, zm), C{t4.re / eps_src, t4.im / eps_src});
      F(s->h_cur, s, 1, ix, iy, zm - 1) = csub(F(s->h_cur, s, 1, ix, iy, zm - 1), rmul(dtcq2 * mu_inv, tf[tfidx(s, 2, ix, iy, zm)]));
      F(s->h_cur, s, 2, ix, iy, zm) = cadd(F(s->h_cur, s, 2, ix, iy, zm), rmul(dtcq2 * mu_inv, tf[tfidx(s, 1, ix, iy, zm)]));
    }
}

// scattering_fourier, code/dataprocess.f90:109-209
static void scattering_fourier(orc_state* s, int nb, int it) {
  const orc_params& p = s->p;
  int nx = s->nx, ny = s->ny;
  bool j_on[3];
  if (ny != 1 && nx != 1) {
    if (p.system_model == 0) { j_on[0] = j_on[1] = j_on[2] = true; }
    else { j_on[0] = j_on[1] = false; j_on[2] = true; }
  } else {
    j_on[0] = (ny == 1 && nx != 1);
    j_on[1] = (nx == 1 && ny != 1);
    j_on[2] = true;
  }
  bool only_e12_h12 = (ny != 1 && nx != 1 && p.system_model != 0);
  for (int j = 0; j < 3; ++j) {
    if (!j_on[j]) continue;
    long n = s->npts[nb][j];
    const int* pt = s->pto[nb][j].data();
    C* fd = s->fdata[nb][j].data();
#pragma omp parallel for num_threads(s->nthreads) schedule(static)
    for (int iw = 0; iw < p.nof; ++iw) {
      double w = s->fw[iw];
      C ph = cexp_i(w * (double)it);  // cdexp(ci*w*it), hoisted out of the point loop
      C* f = fd + (long)iw * n;
      for (long i = 0; i < n; ++i) {
        const int* q = pt + 4 * i;
        int comp = q[0];
        C v;
        if (only_e12_h12) {
          if (comp < 3) v = F(s->e_cur, s, comp, q[1], q[2], q[3]);
          else if (comp > 3 && comp < 6) v = F(s->h_cur, s, comp - 3, q[1], q[2], q[3]);
          else continue;
        } else {
          v = comp < 4 ? F(s->e_cur, s, comp, q[1], q[2], q[3]) : F(s->h_cur, s, comp - 3, q[1], q[2], q[3]);
        }
        f[i] = cadd(f[i], cmul(rmul(p.dt, v), ph));
      }
    }
  }
}

// scattering_fourier_out, flux part: code/dataprocess.f90:243-277.  J is (6, nof), face-major.
void orc_flux(orc_state* s, int nb, double* J) {
  const orc_params& p = s->p;
  int nof = p.nof;
  for (int k = 0; k < 6 * nof; ++k) J[k] = 0.0;
  for (int iw = 0; iw < nof; ++iw)
    for (int j = 0; j < 3; ++j) {
      long n = s->npts[nb][j];
      if (j == 0 && s->nx == 1) continue;
      if (j == 1 && s->ny == 1) continue;
      const C* f = s->fdata[nb][j].data() + (long)iw * n;
      for (long i = 0; i < n; i += 6) {
        auto re_cc = [](C a, C b) { C bc{b.re, -b.im}; return cmul(a, bc); };
        double v;
        if (j == 0) v = csub(re_cc(f[i + 1], f[i + 5]), re_cc(f[i + 2], f[i + 4])).re;
        else if (j == 1) v = csub(re_cc(f[i + 2], f[i + 3]), re_cc(f[i], f[i + 5])).re;
        else v = csub(re_cc(f[i], f[i + 4]), re_cc(f[i + 1], f[i + 3])).re;
        int face = 2 * j + (i + 1 <= n / 2 ? 0 : 1);
        double& acc = J[face * nof + iw];
        if (face % 2 == 0) acc = acc - v; else acc = acc + v;
      }
    }
  double scale = p.eps0 * p.Q / (2.0 * p.dt);
  for (int k = 0; k < 6 * nof; ++k) J[k] = scale * J[k];
}

// One pass of the driver loop body, code/driver.f90:356-451.
static void step(orc_state* s, int it) {
  const orc_params& p = s->p;
  std::swap(s->e_cur, s->e_prev);
  std::swap(s->h_cur, s->h_prev);
  for (int k = 0; k < 2; ++k) {
    std::swap(s->d_cur[k], s->d_prev[k]);
    std::swap(s->b_cur[k], s->b_prev[k]);
  }
  e_fdtd(s);
  upml_e(s);
  bloch_max(s);
  double dtcq2 = (p.dt * p.c0 / p.Q) * (p.dt * p.c0 / p.Q);
  h_fdtd(s, dtcq2);
  upml_h(s);
  bloch_min(s);
  for (auto& v : s->tfsf) v = C{0, 0};
  if (p.plane_wave == 0) tfsf_plane_wave(s, it);
  else if (p.plane_wave == 1) tfsf_gauss(s, it);
  if (s->ny != 1 && s->nx != 1) tfsf_update_3d(s);
  else {
    if (p.i_pol == 2) tfsf_update_2d(s);
    if (p.i_pol == 1) tfsf_update_3d(s);
  }
  if (it >= p.to_fourier && it % p.sample_fourier == 0) {
    scattering_fourier(s, 0, it + 1 - p.to_fourier);
    if (s->nboxes == 2) scattering_fourier(s, 1, it + 1 - p.to_fourier);
  }
}

// Run steps it0..it0+n-1.  If J_out is given, the flux of box 1 is written at
// every output step (code/driver.f90:455-498): J_out[k] holds block k, each
// (6, nof); out_its[k] the step; *nout the number of blocks written.
int orc_run(orc_state* s, int it0, int n, double* J_out, int* out_its, int max_out, int* nout, int* nos_io) {
  const orc_params& p = s->p;
  int nos = nos_io ? *nos_io : 1;
  int k = 0;
  for (int it = it0; it < it0 + n; ++it) {
    step(s, it);
    if (it >= p.to_fourier && (it == p.to_fourier + p.no_downloads * nos || it == p.texit)) {
      if (J_out && k < max_out) {
        orc_flux(s, 0, J_out + (long)k * 6 * p.nof);
        if (out_its) out_its[k] = it;
        ++k;
      }
      ++nos;
    }
  }
  if (nout) *nout = k;
  if (nos_io) *nos_io = nos;
  return 0;
}

// Timed run for the CPU baseline: seconds spent in scattering_fourier and in
// everything else (stencil, UPML, Bloch, TF/SF).
int orc_run_timed(orc_state* s, int it0, int n, double* t_dft, double* t_rest) {
  using clk = std::chrono::steady_clock;
  const orc_params& p = s->p;
  double td = 0.0, tr = 0.0;
  for (int it = it0; it < it0 + n; ++it) {
    auto a = clk::now();
    std::swap(s->e_cur, s->e_prev);
    std::swap(s->h_cur, s->h_prev);
    for (int k = 0; k < 2; ++k) {
      std::swap(s->d_cur[k], s->d_prev[k]);
      std::swap(s->b_cur[k], s->b_prev[k]);
    }
    e_fdtd(s);
    upml_e(s);
    bloch_max(s);
    double dtcq2 = (p.dt * p.c0 / p.Q) * (p.dt * p.c0 / p.Q);
    h_fdtd(s, dtcq2);
    upml_h(s);
    bloch_min(s);
    for (auto& v : s->tfsf) v = C{0, 0};
    if (p.plane_wave == 0) tfsf_plane_wave(s, it);
    else if (p.plane_wave == 1) tfsf_gauss(s, it);
    if (s->ny != 1 && s->nx != 1) tfsf_update_3d(s);
    else {
      if (p.i_pol == 2) tfsf_update_2d(s);
      if (p.i_pol == 1) tfsf_update_3d(s);
    }
    auto b = clk::now();
    if (it >= p.to_fourier && it % p.sample_fourier == 0) {
      scattering_fourier(s, 0, it + 1 - p.to_fourier);
      if (s->nboxes == 2) scattering_fourier(s, 1, it + 1 - p.to_fourier);
    }
    auto c = clk::now();
    tr += std::chrono::duration<double>(b - a).count();
    td += std::chrono::duration<double>(c - b).count();
  }
  *t_dft = td;
  *t_rest = tr;
  return 0;
}

long orc_total_points(orc_state* s) {
  long n = 0;
  for (int b = 0; b < s->nboxes; ++b)
    for (int j = 0; j < 3; ++j) {
      if (j == 0 && s->nx == 1) continue;
      if (j == 1 && s->ny == 1) continue;
      n += s->npts[b][j];
    }
  return n;
}

// Single operators, for per-operator parity (each acts on the current buffers
// without swapping, exactly as the reference subroutine does).
void orc_op_swap(orc_state* s) {
  std::swap(s->e_cur, s->e_prev);
  std::swap(s->h_cur, s->h_prev);
  for (int k = 0; k < 2; ++k) {
    std::swap(s->d_cur[k], s->d_prev[k]);
    std::swap(s->b_cur[k], s->b_prev[k]);
  }
}
void orc_op_e_fdtd(orc_state* s) { e_fdtd(s); }
void orc_op_upml_e(orc_state* s) { upml_e(s); }
void orc_op_bloch_max(orc_state* s) { bloch_max(s); }
void orc_op_h_fdtd(orc_state* s) {
  const orc_params& p = s->p;
  h_fdtd(s, (p.dt * p.c0 / p.Q) * (p.dt * p.c0 / p.Q));
}
void orc_op_upml_h(orc_state* s) { upml_h(s); }
void orc_op_bloch_min(orc_state* s) { bloch_min(s); }
void orc_op_tfsf(orc_state* s, int it) {
  const orc_params& p = s->p;
  for (auto& v : s->tfsf) v = C{0, 0};
  if (p.plane_wave == 0) tfsf_plane_wave(s, it);
  else if (p.plane_wave == 1) tfsf_gauss(s, it);
  if (s->ny != 1 && s->nx != 1) tfsf_update_3d(s);
  else {
    if (p.i_pol == 2) tfsf_update_2d(s);
    if (p.i_pol == 1) tfsf_update_3d(s);
  }
}
void orc_op_dft(orc_state* s, int t) {
  scattering_fourier(s, 0, t);
  if (s->nboxes == 2) scattering_fourier(s, 1, t);
}

// Field access in the reference layout (3, 0:nx+1, 0:ny+1, 0:nz+1), split
// re/im.  which: 0 e_cur, 1 h_cur, 2 e_prev, 3 h_prev.
static C* field_ptr(orc_state* s, int which) {
  switch (which) {
    case 0: return s->e_cur;
    case 1: return s->h_cur;
    case 2: return s->e_prev;
    default: return s->h_prev;
  }
}
void orc_get_field(orc_state* s, int which, double* re, double* im) {
  C* f = field_ptr(s, which);
  long n = 3 * s->sz;
  for (long i = 0; i < n; ++i) { re[i] = f[i].re; im[i] = f[i].im; }
}
void orc_set_field(orc_state* s, int which, const double* re, const double* im) {
  C* f = field_ptr(s, which);
  long n = 3 * s->sz;
  for (long i = 0; i < n; ++i) f[i] = C{re[i], im[i]};
}
// UPML aux: which 0 d, 1 b; cur (1) or prev (0); slab 0 bottom, 1 top.  (3,nx,ny,n)
long orc_pml_size(orc_state* s, int slab) { return 3L * s->nx * s->ny * (slab == 0 ? s->nbot : s->ntop); }
void orc_get_pml(orc_state* s, int which, int cur, int slab, double* re, double* im) {
  C* f = which == 0 ? (cur ? s->d_cur[slab] : s->d_prev[slab]) : (cur ? s->b_cur[slab] : s->b_prev[slab]);
  long n = orc_pml_size(s, slab);
  for (long i = 0; i < n; ++i) { re[i] = f[i].re; im[i] = f[i].im; }
}
void orc_set_pml(orc_state* s, int which, int cur, int slab, const double* re, const double* im) {
  C* f = which == 0 ? (cur ? s->d_cur[slab] : s->d_prev[slab]) : (cur ? s->b_cur[slab] : s->b_prev[slab]);
  long n = orc_pml_size(s, slab);
  for (long i = 0; i < n; ++i) f[i] = C{re[i], im[i]};
}
void orc_get_sz(orc_state* s, double* fpzmn, double* fmzmn, double* fpzmx, double* fmzmx) {
  std::memcpy(fpzmn, s->fpzmn.data(), s->fpzmn.size() * 8);
  std::memcpy(fmzmn, s->fmzmn.data(), s->fmzmn.size() * 8);
  std::memcpy(fpzmx, s->fpzmx.data(), s->fpzmx.size() * 8);
  std::memcpy(fmzmx, s->fmzmx.data(), s->fmzmx.size() * 8);
}
long orc_npts(orc_state* s, int nb, int j) { return s->npts[nb][j]; }
long orc_fdata_len(orc_state* s, int nb, int j) { return (long)s->fdata[nb][j].size(); }
// fdata(i_pts, iw), i_pts fastest: re/im of length orc_fdata_len
void orc_get_fdata(orc_state* s, int nb, int j, double* re, double* im) {
  const std::vector<C>& f = s->fdata[nb][j];
  for (size_t i = 0; i < f.size(); ++i) { re[i] = f[i].re; im[i] = f[i].im; }
}
void orc_get_pto(orc_state* s, int nb, int j, int* out) {
  std::memcpy(out, s->pto[nb][j].data(), s->pto[nb][j].size() * sizeof(int));
}
// tfsf_data after the last orc_op_tfsf / step: (6, nx+4, ny+4, nzt) split re/im
long orc_tfsf_len(orc_state* s) { return (long)s->tfsf.size(); }
void orc_get_tfsf(orc_state* s, double* re, double* im) {
  for (size_t i = 0; i < s->tfsf.size(); ++i) { re[i] = s->tfsf[i].re; im[i] = s->tfsf[i].im; }
}

// spectra_lossless_dielectric, code/common.f90:104-131: analytic R,T of the film.
void orc_film_spectrum(const orc_params* p, double lno, double dlamda, int dh, int nwo, int nwf,
                       double* lp_out, double* R_out, double* T_out) {
  C nII = {std::sqrt(p->eps_bbox_re), 0.0};  // real eps_bbox here
  C nIII = {std::sqrt(p->eps3), 0.0};
  for (int iw = nwo; iw <= nwf; ++iw) {
    double lp = lno + dlamda * ((double)iw - 1.0);
    double del = 2 * p->pi * nII.re * (double)dh * p->Q / (lp * p->f_abohr);
    double cd = std::cos(del), sd = std::sin(del);
    C ci{0.0, 1.0};
    C r32 = cdiv(nIII, nII);
    C a = cadd(C{cd, 0.0}, cmul(rmul(sd, r32), ci));
    C b = cadd(rmul(cd, nIII), cmul(ci, rmul(sd, nII)));
    C num = csub(a, b);
    C den = cadd(a, b);
    C cn = cdiv(num, den);
    C cc{cn.re, -cn.im};
    C m = cmul(cc, cn);
    double R = std::sqrt(m.re * m.re + m.im * m.im);
    lp_out[iw - nwo] = lp;
    R_out[iw - nwo] = R;
    T_out[iw - nwo] = 1.0 - R;
  }
}

}  // extern "C"
