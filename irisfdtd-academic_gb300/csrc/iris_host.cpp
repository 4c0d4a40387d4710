// Host side of the GB300 FDTD engine: the inputFDTD.dat reader (setparam),
// the physical constants, the output writers and the drop-in main program
// (program IrisFDTD -> main -> driver) on top of the C ABI.
#include <cerrno>
#include <chrono>
#include <cmath>
#include <ctime>
#include <complex>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "iris_internal.h"

using iris::fail;

namespace {

// ---------------------------------------------------------------------------
// Fortran list-directed input: a read of n items takes the leading values of
// the next record, continuing on following records until n values are found;
// the rest of the last record is skipped.  Values are separated by blanks,
// tabs or commas; '/' ends the read; quoted strings and parenthesised
// complex constants are single values.

struct Tok {
  enum Kind { WORD, STR, CPLX, SLASH } kind;
  std::string text;
};

class ListReader {
 public:
  explicit ListReader(std::vector<std::string> lines) : lines_(std::move(lines)) {}
  void rewind() { pos_ = 0; }
  bool eof() const { return pos_ >= lines_.size(); }
  // false at end of file
  bool read(size_t n, std::vector<Tok>& out) {
    out.clear();
    while (out.size() < n) {
      if (eof()) return false;
      std::vector<Tok> t = split(lines_[pos_++]);
      for (const Tok& k : t) {
        if (k.kind == Tok::SLASH) {
          while (out.size() < n) out.push_back(Tok{Tok::WORD, ""});
          return true;
        }
        out.push_back(k);
        if (out.size() == n) break;
      }
    }
    return true;
  }

 private:
  static std::vector<Tok> split(const std::string& s) {
    std::vector<Tok> out;
    size_t i = 0, n = s.size();
    auto sep = [](char c) { return c == ' ' || c == '\t' || c == '\r' || c == '\n' || c == ','; };
    while (i < n) {
      const char c = s[i];
      if (sep(c)) { ++i; continue; }
      if (c == '/') { out.push_back({Tok::SLASH, "/"}); break; }
      if (c == '\'' || c == '"') {
        size_t j = s.find(c, i + 1);
        if (j == std::string::npos) j = n;
        out.push_back({Tok::STR, s.substr(i + 1, j - i - 1)});
        i = j + 1;
        continue;
      }
      if (c == '(') {
        size_t j = s.find(')', i);
        if (j == std::string::npos) j = n;
        out.push_back({Tok::CPLX, s.substr(i + 1, j - i - 1)});
        i = j + 1;
        continue;
      }
      size_t j = i;
      while (j < n && !sep(s[j]) && s[j] != '/') ++j;
      out.push_back({Tok::WORD, s.substr(i, j - i)});
      i = j;
    }
    return out;
  }
  std::vector<std::string> lines_;
  size_t pos_ = 0;
};

bool to_int(const Tok& t, int& v) {
  if (t.kind != Tok::WORD || t.text.empty()) return false;
  char* end = nullptr;
  errno = 0;
  long x = std::strtol(t.text.c_str(), &end, 10);
  if (errno || *end != '\0') return false;
  v = (int)x;
  return true;
}

bool to_real_str(std::string s, double& v) {
  for (char& c : s)
    if (c == 'd' || c == 'D') c = 'e';
  if (s.empty()) return false;
  char* end = nullptr;
  errno = 0;
  v = std::strtod(s.c_str(), &end);
  return !errno && *end == '\0';
}

bool to_real(const Tok& t, double& v) { return t.kind == Tok::WORD && to_real_str(t.text, v); }

bool to_complex(const Tok& t, double& re, double& im) {
  if (t.kind == Tok::CPLX) {
    size_t k = t.text.find(',');
    if (k == std::string::npos) return false;
    std::string a = t.text.substr(0, k), b = t.text.substr(k + 1);
    auto trim = [](std::string x) {
      size_t i = x.find_first_not_of(" \t"), j = x.find_last_not_of(" \t");
      return i == std::string::npos ? std::string() : x.substr(i, j - i + 1);
    };
    return to_real_str(trim(a), re) && to_real_str(trim(b), im);
  }
  im = 0.0;
  return to_real(t, re);
}

// struct_limit, code/files.f90:385-409
void struct_limit(int N, int a, int& ai, int& af) {
  if (a % 2 == 0) {
    if (N % 2 == 0) { ai = N / 2 - (a / 2 - 1); af = N / 2 + (a / 2); }
    else { ai = (N + 1) / 2 - a / 2; af = (N + 1) / 2 + a / 2 - 1; }
  } else {
    if (N % 2 == 0) { ai = N / 2 - ((a + 1) / 2 - 1); af = N / 2 + ((a - 1) / 2); }
    else { ai = (N + 1) / 2 - (a - 1) / 2; af = (N + 1) / 2 + (a - 1) / 2; }
  }
}

}  // namespace

extern "C" {

const char* iris_strerror(int status) {
  switch (status) {
    case IRIS_OK: return "success";
    case IRIS_EINVAL: return "invalid argument";
    case IRIS_ENOMEM: return "out of memory";
    case IRIS_ECUDA: return "CUDA error";
    case IRIS_EPARSE: return "invalid input file";
    case IRIS_EIO: return "I/O error";
    case IRIS_ENAN: return "non-finite value";
    case IRIS_ETIMEOUT: return "device wait timed out";
    case IRIS_ENODEV: return "no CUDA device";
    default: return "unknown error";
  }
}

// code/physconst.f90:31-53.  Unsuffixed literals are default REAL: rounded to
// single precision first, then widened.
void iris_physconsts(iris_params* p, int single_literals) {
  if (single_literals) {
    p->pi = (double)(float)3.14159265358979323846;
    p->c0 = (double)137.0360f;
    p->f_abohr = (double)((float)10 / 0.529177249f);
    p->uat = (double)24.188843265E-3f;
    p->f_e = (double)514.2208281e9f;
    p->pmlalfa = (double)1.8f;
  } else {
    p->pi = 3.14159265358979323846;
    p->c0 = 137.0360;
    p->f_abohr = 10 / 0.529177249;
    p->uat = 24.188843265E-3;
    p->f_e = 514.2208281e9;
    p->pmlalfa = 1.8;
  }
  p->eps0 = 1.0 / (4.0 * p->pi);
  p->mu0 = 1.0 / (p->eps0 * (p->c0 * p->c0));
}

int iris_frequencies(const iris_params* p, double* fw, int fw_cap) {
  if (!p || !fw || fw_cap < p->nof) return fail(IRIS_EINVAL, "fw buffer too small");
  double lno_aux = p->lno;
  for (int i = 0; i < p->nof; ++i) {
    fw[i] = 2.0 * p->pi * p->c0 * p->dt / (p->f_abohr * lno_aux);
    lno_aux = lno_aux + p->dlamda;
  }
  return IRIS_OK;
}

int iris_setparam(const char* path, int single_literals, iris_params* out, double* fw, int fw_cap, char* desc,
                  int desc_cap) {
  iris::clear_error();
  if (!path || !out) return fail(IRIS_EINVAL, "null argument");
  std::ifstream in(path);
  if (!in) return fail(IRIS_EPARSE, std::string("cannot open ") + path);
  std::vector<std::string> lines;
  for (std::string l; std::getline(in, l);) lines.push_back(l);
  if (desc && desc_cap > 0) {
    std::string d = lines.empty() ? "" : lines[0].substr(0, 100);
    std::snprintf(desc, desc_cap, "%s", d.c_str());
  }
  iris_params p;
  std::memset(&p, 0, sizeof(p));
  iris_physconsts(&p, single_literals);
  ListReader R(lines);
  std::vector<Tok> t;
  auto perr = [](const std::string& m) { return fail(IRIS_EPARSE, "invalid input file: " + m); };
  // seek a quoted section header by reading the first value of each record
  auto seek = [&](const char* header, bool guarded) {
    R.rewind();
    while (true) {
      if (guarded && R.eof()) return false;
      if (!R.read(1, t)) return false;
      if (t[0].text == header) return true;
    }
  };
  auto rd_int = [&](int& v) { return R.read(1, t) && to_int(t[0], v); };
  auto rd_real = [&](double& v) { return R.read(1, t) && to_real(t[0], v); };

  // 'Mesh options', code/files.f90:48-115
  if (!seek("Mesh options", false)) return perr("no 'Mesh options'");
  if (!rd_int(p.i_pol) || p.i_pol < 1 || p.i_pol > 4) return perr("i_pol");
  if (!rd_real(p.q_nm) || p.q_nm <= 0) return perr("q");
  if (!rd_int(p.nx) || p.nx < 1) return perr("ixmax");
  if (!rd_int(p.ny) || p.ny < 1) return perr("iymax");
  if (!rd_int(p.nz) || p.nz < 1) return perr("izmax");
  p.Q = p.f_abohr * p.q_nm;
  if (!rd_real(p.cfl) || p.cfl <= 0) return perr("CFL");
  p.dt = p.cfl / (p.c0 * std::sqrt(3.0 / (p.Q * p.Q)));
  if (!(p.dt > 0)) return perr("dt");
  if (!rd_real(p.wzpml) || p.wzpml < 0) return perr("wzPML");
  p.wzpml = p.f_abohr * (p.wzpml / p.Q);
  if (!rd_int(p.pml_taflove)) return perr("nPML line");
  p.npml = 2;
  if (!rd_int(p.pmlzi)) return perr("pmlzi");
  if (!rd_int(p.pmlzf)) return perr("pmlzf");

  // 'Job options', code/files.f90:118-154
  if (!seek("Job options", false)) return perr("no 'Job options'");
  int ndl = 0;
  if (!R.read(2, t) || !to_int(t[0], ndl) || !to_int(t[1], p.output_time_step)) return perr("no_downloads");
  if (!rd_real(p.texit_fs)) return perr("itmax");
  p.texit = (int)(p.texit_fs / (p.dt * p.uat));
  if (ndl == 0) return perr("no_downloads = 0");
  p.no_downloads = p.texit / ndl;
  if (!rd_int(p.hi)) return perr("hi");
  if (!R.read(3, t) || !to_int(t[0], p.sdl_plane_on[0]) || !to_int(t[1], p.sdl_plane_on[1]) ||
      !to_int(t[2], p.sdl_plane_on[2]))
    return perr("SDL planes");

  // 'Dielectric constants', code/files.f90:156-170
  if (!seek("Dielectric constants", false)) return perr("no 'Dielectric constants'");
  if (!rd_real(p.eps1)) return perr("eps cover");
  if (!R.read(1, t) || !to_complex(t[0], p.eps_bbox_re, p.eps_bbox_im)) return perr("eps_bbox");
  if (!rd_real(p.eps3)) return perr("eps substrate");

  // 'Fourier transformation options', code/files.f90:173-253
  if (!seek("Fourier transformation options", true)) return perr("no 'Fourier transformation options'");
  for (int k = 0; k < 6; ++k)
    if (!R.read(2, t) || !to_int(t[0], p.box1[k]) || !to_int(t[1], p.box2[k])) return perr("DFT box");
  if (!rd_int(p.nof) || p.nof < 1) return perr("nof");
  if (!rd_real(p.dlamda)) return perr("dlambda");
  if (!rd_real(p.lno)) return perr("lno");
  if (!R.read(2, t) || !to_int(t[0], p.to_fourier) || !to_int(t[1], p.sample_fourier)) return perr("to_Fourier");

  // 'Source options', code/files.f90:256-289
  if (!seek("Source options", true)) return perr("no 'Source options'");
  if (!rd_int(p.plane_wave)) return perr("plane_wave");
  if (!R.read(2, t) || !to_real(t[0], p.tincr) || !to_real(t[1], p.tdecay)) return perr("tincr/tdecay");
  if (!R.read(4, t) || !to_real(t[0], p.epump) || !to_real(t[1], p.wlpump) || !to_real(t[2], p.pump_dt) ||
      !to_real(t[3], p.def_pulse))
    return perr("Epump line");
  if (!rd_int(p.tfsf_zi)) return perr("tfsf_zi");
  p.tfsf_zf = p.tfsf_zi + 5;
  if (!rd_int(p.cosine)) return perr("cosine");
  p.ratio_angle = 1.0;
  p.tincr = p.tincr / p.uat;
  p.tdecay = p.tdecay / p.uat;
  p.epump = p.epump / (p.f_e * (single_literals ? (double)1e-5f : 1e-5));
  p.pump_dt = p.pump_dt / p.uat;
  p.gpump = p.c0 * p.pump_dt / (2.0 * p.Q * std::sqrt(p.eps1 * p.def_pulse));
  p.zopump = -(std::sqrt(p.def_pulse) * p.gpump) - p.tfsf_zi;
  p.gap = 0.0;

  // 'Slit Array', code/files.f90:322-342
  if (!seek("Slit Array", false)) return perr("no 'Slit Array'");
  if (!rd_int(p.dh)) return perr("Dh");
  p.hf = (p.hi + p.dh) - 1;
  if (!rd_int(p.dx)) return perr("dx");
  struct_limit(p.nx, p.dx, p.aix, p.afx);

  p.precision = IRIS_FP64;
  p.dft_block = 0;
  p.device = 0;
  *out = p;
  if (fw) {
    if (fw_cap < p.nof) return fail(IRIS_EINVAL, "fw buffer too small");
    iris_frequencies(&p, fw, fw_cap);
  }
  return IRIS_OK;
}

int iris_write_scatt(const char* dir, int box, int it, int nof, const double* J) {
  if (!dir || !J || nof < 1) return fail(IRIS_EINVAL, "bad argument");
  const std::string base = std::string(dir) + "/" + std::to_string(box + 1) + "_scatt";
  for (int j = 0; j < 6; ++j) {
    FILE* f = std::fopen((base + std::to_string(j + 1) + ".dat").c_str(), "a");
    if (!f) return fail(IRIS_EIO, "cannot open " + base + std::to_string(j + 1) + ".dat");
    std::fprintf(f, " #  %10d\n", it);
    for (int iw = 0; iw < nof; ++iw) std::fprintf(f, "  %24.16E\n", J[j * nof + iw]);
    std::fclose(f);
  }
  FILE* f = std::fopen((base + ".dat").c_str(), "a");
  if (!f) return fail(IRIS_EIO, "cannot open " + base + ".dat");
  std::fprintf(f, " #  %10d\n", it);
  for (int iw = 0; iw < nof; ++iw) {
    const double s = J[0 * nof + iw] + J[1 * nof + iw] + J[2 * nof + iw] + J[3 * nof + iw] + J[4 * nof + iw] +
                     J[5 * nof + iw];
    std::fprintf(f, "  %24.16E\n", s);
  }
  std::fclose(f);
  return IRIS_OK;
}

}  // extern "C"

namespace {

// spectra_lossless_dielectric, code/common.f90:104-131
void write_film_spectrum(const std::string& dir, const iris_params& p) {
  FILE* f = std::fopen((dir + "/dielectric_layer_spectra.dat").c_str(), "w");
  if (!f) return;
  const std::complex<double> nII = std::sqrt(std::complex<double>(p.eps_bbox_re, p.eps_bbox_im));
  const std::complex<double> nIII = std::sqrt(std::complex<double>(p.eps3, 0.0));
  const std::complex<double> ci(0.0, 1.0);
  for (int iw = 1; iw <= p.nof; ++iw) {
    const double lp = p.lno + p.dlamda * (iw - 1.0);
    const double del = (2 * p.pi * nII * (double)p.dh * p.Q / (lp * p.f_abohr)).real();
    const double c = std::cos(del), s = std::sin(del);
    std::complex<double> cn = (c + ci * (nIII / nII) * s - nIII * c - ci * nII * s);
    cn = cn / (c + ci * (nIII / nII) * s + nIII * c + ci * nII * s);
    const double R = std::abs(std::conj(cn) * cn);
    std::fprintf(f, "  %24.16E  %24.16E  %24.16E\n", lp, R, 1.0 - R);
  }
  std::fclose(f);
}

// ---------------------------------------------------------------------------
// SDL field snapshots (code/sdl.f90): the parameters of setparam_SDL
// (:365-400) and of the optional "Extra parameters-SDLextended" section
// (code/files.f90:291-320), and SDL_output's files (:68-234).

struct SdlParams {
  int copy_flag = 0, copy_no = 1;
  int xi[3] = {}, xf[3] = {}, yi[3] = {}, yf[3] = {}, zi[3] = {}, zf[3] = {};
  int module_e = 0;     // 1: |E| from E, 2: |H| from the previous step's H
  int field[6] = {};    // Ex Ey Ez Hx Hy Hz: 1 Re, 2 Im, 3 modulus, 4 |Re|, 5 |Im|
  std::vector<int> delta[3] = {{0}, {0}, {0}};  // extra layers per plane
  bool extended() const { return delta[0].size() != 1 || delta[1].size() != 1 || delta[2].size() != 1; }
  bool wants_e() const { return module_e == 1 || field[0] >= 1 || field[1] >= 1 || field[2] >= 1; }
  bool wants_h() const { return module_e == 2 || field[3] >= 1 || field[4] >= 1 || field[5] >= 1; }
};

int read_sdl(const std::string& path, SdlParams& q) {
  std::ifstream in(path);
  std::vector<std::string> lines;
  for (std::string l; std::getline(in, l);) lines.push_back(l);
  ListReader R(lines);
  std::vector<Tok> t;
  auto seek = [&](const char* header) {
    R.rewind();
    while (!R.eof()) {
      if (!R.read(1, t)) return false;
      if (t[0].text == header) return true;
    }
    return false;
  };
  auto perr = [](const std::string& m) { return fail(IRIS_EPARSE, "invalid SDL section: " + m); };
  if (!seek("Time evolution options")) return perr("no 'Time evolution options'");
  if (!R.read(2, t) || !to_int(t[0], q.copy_flag) || !to_int(t[1], q.copy_no)) return perr("SDL_copy_flag");
  int* rows[6] = {q.xi, q.xf, q.yi, q.yf, q.zi, q.zf};
  for (int r = 0; r < 6; ++r)
    if (!R.read(3, t) || !to_int(t[0], rows[r][0]) || !to_int(t[1], rows[r][1]) || !to_int(t[2], rows[r][2]))
      return perr("plane ranges");
  if (!R.read(1, t) || !to_int(t[0], q.module_e)) return perr("SDLModuleE");
  for (int k = 0; k < 6; ++k)
    if (!R.read(1, t) || !to_int(t[0], q.field[k])) return perr("SDLField");
  if (seek("Extra parameters-SDLextended")) {
    int n[3];
    if (!R.read(3, t) || !to_int(t[0], n[0]) || !to_int(t[1], n[1]) || !to_int(t[2], n[2])) return perr("extra layers");
    for (int a = 0; a < 3; ++a) {
      if (n[a] < 1) return perr("extra layers must be >= 1");
      q.delta[a].assign(n[a], 0);
      for (int i = 0; i < n[a]; ++i)
        if (!R.read(1, t) || !to_int(t[0], q.delta[a][i])) return perr("layer offsets");
    }
  }
  if (q.copy_flag && q.copy_no < 1) return perr("SDL_copy_no");
  return IRIS_OK;
}

// inttoASCII (code/common.f90:40-101): plain decimal digits
std::string sdl_number(int n) { return std::to_string(n); }

// One plane request: layer 1, 2, 3 (x, y, z = const), its index and ranges.
struct SdlPlane {
  int layer, index, lo1, hi1, lo2, hi2;
};

std::vector<SdlPlane> sdl_planes(const iris_params& p, const SdlParams& q) {
  std::vector<SdlPlane> out;
  for (int l = 1; l <= 3; ++l) {
    if (!p.sdl_plane_on[l - 1]) continue;
    for (int d : q.delta[l - 1]) {
      const int j = l - 1;
      if (l == 1) out.push_back({1, q.xi[j] + d, q.yi[j], q.yf[j], q.zi[j], q.zf[j]});
      if (l == 2) out.push_back({2, q.yi[j] + d, q.xi[j], q.xf[j], q.zi[j], q.zf[j]});
      if (l == 3) out.push_back({3, q.zi[j] + d, q.xi[j], q.xf[j], q.yi[j], q.yf[j]});
    }
  }
  return out;
}

// One Fortran unformatted sequential record of REAL(4) values.
int write_record(const std::string& path, const std::vector<float>& v) {
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) return fail(IRIS_EIO, "cannot write " + path);
  const uint32_t n = (uint32_t)(v.size() * 4);
  bool ok = std::fwrite(&n, 4, 1, f) == 1;
  ok = ok && (v.empty() || std::fwrite(v.data(), 4, v.size(), f) == v.size());
  ok = ok && std::fwrite(&n, 4, 1, f) == 1;
  ok = (std::fclose(f) == 0) && ok;
  return ok ? IRIS_OK : fail(IRIS_EIO, "write failed: " + path);
}

// SDL_output for one plane and one quantity: em 0 (modulus of all three
// components), 1 (a component of E), 2 (a component of H); comp 0..2; the
// plane's values re/im (component fastest) as iris_get_plane returns them.
int sdl_output(const std::string& dir, const iris_params& p, const SdlParams& q, const SdlPlane& pl, int nos, int em,
               int comp, int mode, bool module_h, const std::vector<double>& re, const std::vector<double>& im) {
  const int n1 = pl.hi1 - pl.lo1 + 1, n2 = pl.hi2 - pl.lo2 + 1;
  std::string ext, ext2;
  if (em == 0) {
    ext = ".e";
    ext2 = module_h ? "_H" : "_E";
  } else {
    ext = std::string(em == 1 ? ".e" : ".h") + char('1' + comp);
    static const char* m[6] = {"", "_R", "_I", "_MC", "_MR", "_MI"};
    ext2 = mode >= 1 && mode <= 5 ? m[mode] : "";
  }
  static const char* axis_name[4] = {"", "X", "Y", "Z"};
  std::string name = std::string("/") + axis_name[pl.layer] + "_SDL";
  if (q.extended()) name += sdl_number(pl.index) + "layer";
  name += ext2 + sdl_number(nos) + ext;
  // Output(i1, i2), i1 fastest; values / (q * Epump) (the TF/SF amplitude)
  double norm = p.Q * p.epump;
  if (norm == 0.0) norm = 1.0;
  std::vector<double> out((size_t)n1 * n2);
  for (int b = 0; b < n2; ++b)
    for (int a = 0; a < n1; ++a) {
      const size_t c = (size_t)b * n1 + a;
      double v = 0.0;
      if (em == 0) {
        double s = 0.0;
        for (int k = 0; k < 3; ++k) s += re[3 * c + k] * re[3 * c + k] + im[3 * c + k] * im[3 * c + k];
        v = std::sqrt(s);
      } else {
        const double r = re[3 * c + comp], i = im[3 * c + comp];
        switch (mode) {
          case 1: v = r; break;
          case 2: v = i; break;
          case 3: v = std::sqrt(r * r + i * i); break;
          case 4: v = std::sqrt(r * r); break;
          case 5: v = std::sqrt(i * i); break;
          default: v = 0.0;
        }
      }
      // output = real(output)/SDLnorm (code/sdl.f90:363): rounded to REAL(4),
      // divided in REAL(8), written as REAL(4) (:449-456)
      out[c] = (double)(float)v / norm;
    }
  std::vector<float> rec;
  if (q.copy_flag) {
    // output_aux(ixo : copies*(ixf+1-ixo), iyo : ...) filled at ix + i*(ixf+1-ixo)
    // (and, for z planes, iy + j*(iyf+1-iyo)); cells the copies do not reach
    // (lower bounds below 1) are left 0 here
    const int c1 = q.copy_no, c2 = pl.layer == 3 ? q.copy_no : 1;
    const int m1 = c1 * (pl.hi1 + 1 - pl.lo1) - pl.lo1 + 1, m2 = pl.layer == 3 ? c2 * (pl.hi2 + 1 - pl.lo2) - pl.lo2 + 1 : n2;
    rec.assign((size_t)std::max(m1, 0) * std::max(m2, 0), 0.0f);
    for (int j = 0; j < c2; ++j)
      for (int i = 0; i < c1; ++i)
        for (int b = 0; b < n2; ++b)
          for (int a = 0; a < n1; ++a) {
            const int x = a + i * n1, y = b + j * n2;  // offsets from (lo1, lo2)
            if (x < m1 && y < m2) rec[(size_t)y * m1 + x] = (float)out[(size_t)b * n1 + a];
          }
  } else {
    rec.assign(out.begin(), out.end());
  }
  return write_record(dir + name, rec);
}

// setSDL_FILE (code/sdl.f90:404-448) for one plane: E quantities from e (the
// current E), H quantities from h (the H of the step before).  SDLField(4:6)
// switch the H components on, but SDL_output takes the mode (and the name's
// suffix) of component k from SDLField(k), the E entry (:140-153, :202-212);
// with no mode there the name has no suffix and the values are left
// unassigned by the reference (0 here).
int sdl_files(const std::string& dir, const iris_params& p, const SdlParams& q, const SdlPlane& pl, int nos,
              const std::vector<double>& ere, const std::vector<double>& eim, const std::vector<double>& hre,
              const std::vector<double>& him) {
  int rc = IRIS_OK;
  if (q.module_e == 1) rc = sdl_output(dir, p, q, pl, nos, 0, 0, 0, false, ere, eim);
  if (!rc && q.module_e == 2) rc = sdl_output(dir, p, q, pl, nos, 0, 0, 0, true, hre, him);
  for (int k = 0; k < 3 && !rc; ++k)
    if (q.field[k] >= 1) rc = sdl_output(dir, p, q, pl, nos, 1, k, q.field[k], false, ere, eim);
  for (int k = 0; k < 3 && !rc; ++k)
    if (q.field[3 + k] >= 1) rc = sdl_output(dir, p, q, pl, nos, 2, k, q.field[k], false, hre, him);
  return rc;
}

int get_planes(iris_engine* eng, int which, const std::vector<SdlPlane>& pls, std::vector<std::vector<double>>& re,
               std::vector<std::vector<double>>& im) {
  re.resize(pls.size());
  im.resize(pls.size());
  for (size_t i = 0; i < pls.size(); ++i) {
    const SdlPlane& pl = pls[i];
    const size_t m = 3 * (size_t)(pl.hi1 - pl.lo1 + 1) * (pl.hi2 - pl.lo2 + 1);
    re[i].resize(m);
    im[i].resize(m);
    int rc = iris_get_plane(eng, which, pl.layer, pl.index, pl.lo1, pl.hi1, pl.lo2, pl.hi2, re[i].data(), im[i].data());
    if (rc) return rc;
  }
  return IRIS_OK;
}

// main() + driver(), code/main.f90:43-213 and code/driver.f90:66-555; loop:
// called from the <<LOOP>> mode, whose main(i) logs an empty description
// (code/main.f90:108-113)
int run_main(const std::string& dir, int precision, bool loop = false) {
  iris_params p;
  char desc[128] = {0};
  int rc = iris_setparam((dir + "/inputFDTD.dat").c_str(), 1, &p, nullptr, 0, desc, sizeof(desc));
  if (rc) return rc;
  if (loop) desc[0] = 0;
  p.precision = precision;
  std::vector<double> fw(p.nof);
  iris_frequencies(&p, fw.data(), p.nof);
  FILE* log = std::fopen((dir + "/log.dat").c_str(), "w");
  if (!log) return fail(IRIS_EIO, "cannot write log.dat");
  std::fprintf(log, " Description     : %s\n", desc);
  std::fprintf(log, "# q(nm)=%15.5f q(u.a)=%15.5f\n", p.q_nm, p.Q);
  std::fprintf(log, "# ixmax=%d iymax=%d izmax=%d\n", p.nx, p.ny, p.nz);
  std::fprintf(log, "# CFL =%15.5f\n", p.cfl);
  std::fprintf(log, "# dt(fs)=%15.8f\n", p.dt * p.uat);
  std::fprintf(log, "# Iteration max. number = %d Simulation time = %15.5f (fs)\n", p.texit, p.uat * p.dt * p.texit);
  std::fprintf(log, "# pmlzi=%d pmlzf=%d hi=%d hf=%d aix=%d afx=%d\n", p.pmlzi, p.pmlzf, p.hi, p.hf, p.aix, p.afx);
  std::fprintf(log, "# precision=%s\n", precision == IRIS_FP64 ? "fp64" : "fp32");
  write_film_spectrum(dir, p);
  const bool sdl_on = p.sdl_plane_on[0] || p.sdl_plane_on[1] || p.sdl_plane_on[2];
  SdlParams sdl;
  std::vector<SdlPlane> planes;
  if (sdl_on) {
    rc = read_sdl(dir + "/inputFDTD.dat", sdl);
    if (rc) { std::fclose(log); return rc; }
    planes = sdl_planes(p, sdl);
    std::fprintf(log, "#SDL planes=%d (x %d, y %d, z %d)\n", (int)planes.size(), p.sdl_plane_on[0], p.sdl_plane_on[1],
                 p.sdl_plane_on[2]);
  }
  const bool sdl_h = sdl_on && sdl.wants_h();
  std::vector<std::vector<double>> ere, eim, hre, him;
  iris_engine* eng = nullptr;
  rc = iris_create(&p, fw.data(), &eng);
  if (rc) { std::fclose(log); return rc; }
  bool single = true;
  for (int i = 0; i < 6; ++i)
    if (p.box1[i] != p.box2[i]) single = false;
  std::vector<double> J(6 * (size_t)p.nof);
  int nos = 1;
  // the screen progress of code/driver.f90:339-354 (date, iteration, rate,
  // time left, share done) every OUTPUT_TIME_STEP steps, printed at the next
  // point where the host waits for the device anyway (an output step), with
  // the rate measured over the steps since the last line; IRIS_QUIET=1
  // silences it
  const bool quiet = std::getenv("IRIS_QUIET") && std::string(std::getenv("IRIS_QUIET")) == "1";
  auto last_t = std::chrono::steady_clock::now();
  int last_it = 0;
  auto progress = [&](int at) {
    if (quiet || p.output_time_step <= 0 || at / p.output_time_step == last_it / p.output_time_step) return;
    const auto now = std::chrono::steady_clock::now();
    const double sec = std::chrono::duration<double>(now - last_t).count();
    const double rate = sec > 0 ? (at - last_it) / sec : 0.0;
    const std::time_t tt = std::time(nullptr);
    char date[32];
    std::strftime(date, sizeof date, "%d/%m/%Y-%H:%M:%S", std::localtime(&tt));
    std::printf("  Date = %s\n  Iteration %d of %d\n  Iteration/second = %.3f\n  Finish in %.6f hours\n"
                "  Completed %.3f %%\n",
                date, at, p.texit, rate, rate > 0 ? (p.texit - at) / rate / 3600.0 : 0.0, 100.0 * at / p.texit);
    std::fflush(stdout);
    last_t = now;
    last_it = at;
  };
  // step in chunks that end at output steps
  int it = 1;
  while (it <= p.texit && rc == IRIS_OK) {
    int next = p.texit;
    if (p.to_fourier + p.no_downloads * nos >= it && p.to_fourier + p.no_downloads * nos < next)
      next = p.to_fourier + p.no_downloads * nos;
    if (next < it) next = it;
    const bool output = next >= p.to_fourier && (next == p.to_fourier + p.no_downloads * nos || next == p.texit);
    if (output && sdl_h) {
      // the SDL's H is h_prev: the H of the step before the output step
      if (next > it) rc = iris_step(eng, it, next - it);
      if (!rc) rc = get_planes(eng, IRIS_H, planes, hre, him);
      if (!rc) rc = iris_step(eng, next, 1);
    } else {
      rc = iris_step(eng, it, next - it + 1);
    }
    if (rc) break;
    it = next;
    if (output && sdl_on) {
      rc = get_planes(eng, IRIS_E, planes, ere, eim);
      // the driver numbers the snapshot files nos + 1 (code/driver.f90:473-491)
      for (size_t i = 0; i < planes.size() && !rc; ++i)
        rc = sdl_files(dir, p, sdl, planes[i], nos + 1, ere[i], eim[i], sdl_h ? hre[i] : ere[i],
                       sdl_h ? him[i] : eim[i]);
      if (rc) break;
    }
    if (it >= p.to_fourier && (it == p.to_fourier + p.no_downloads * nos || it == p.texit)) {
      rc = iris_flux(eng, 0, J.data());
      if (rc == IRIS_OK || rc == IRIS_ENAN) rc = iris_write_scatt(dir.c_str(), 0, it, p.nof, J.data()) ? IRIS_EIO : rc;
      if (!single && rc == IRIS_OK) {
        rc = iris_flux(eng, 1, J.data());
        if (rc == IRIS_OK) rc = iris_write_scatt(dir.c_str(), 1, it, p.nof, J.data());
      }
      ++nos;
      progress(it);
    }
    ++it;
  }
  if (rc == IRIS_OK) rc = iris_sync(eng);
  std::fprintf(log, " ...done! status=%d\n", rc);
  std::fclose(log);
  iris_destroy(eng);
  return rc;
}

}  // namespace

extern "C" int iris_run_input(const char* dir, int precision) {
  iris::clear_error();
  if (!dir) return fail(IRIS_EINVAL, "null directory");
  const std::string d(dir);
  std::ifstream in(d + "/inputFDTD.dat");
  if (!in) return fail(IRIS_EPARSE, "cannot open " + d + "/inputFDTD.dat");
  std::string first;
  std::getline(in, first);
  if (first.rfind("<<LOOP>>", 0) != 0) return run_main(d, precision);
  // program.f90:40-57: io_main, if_main, delta_x, delta_y, delta_z
  std::vector<std::string> rest;
  for (std::string l; std::getline(in, l);) rest.push_back(l);
  ListReader R(rest);
  std::vector<Tok> t;
  int io = 0, ifm = 0;
  if (!R.read(1, t) || !to_int(t[0], io) || !R.read(1, t) || !to_int(t[0], ifm))
    return fail(IRIS_EPARSE, "invalid <<LOOP>> header");
  int rc = IRIS_OK;
  if (io != ifm) {
    for (int i = io; i <= ifm && rc == IRIS_OK; ++i) rc = run_main(d, precision, true);
  } else {
    rc = run_main(d, precision, true);
  }
  return rc;
}
