// Engine internals shared by the CUDA translation units (iris_engine.cu,
// iris_batch.cu, iris_adjoint.cu): the engine state and the host helpers
// that build its kernel arguments, flush its DFT ring and replay its graphs.
// Not part of the public ABI.
#pragma once
#include <cuda_runtime.h>

#include <functional>
#include <string>
#include <utility>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "iris_device.cuh"
#include "iris_internal.h"

// Return IRIS_ECUDA (IRIS_ENOMEM for an allocation) with the failing call's
// text when a CUDA runtime call fails.
#define CK(call)                                                                        \
  do {                                                                                  \
    cudaError_t err_ = (call);                                                          \
    if (err_ != cudaSuccess)                                                            \
      return iris::fail(err_ == cudaErrorMemoryAllocation ? IRIS_ENOMEM : IRIS_ECUDA,   \
                        std::string(#call) + ": " + cudaGetErrorString(err_));          \
  } while (0)

namespace iris {

struct FaceMap {
  bool active = false;  // this face pair is accumulated by scattering_fourier
  int nu = 0, nv = 0;
  long nloc = 0;         // locations per face
  long base[2][6] = {};  // first sample index per [side][component]
};

}  // namespace iris

struct iris_engine {
  iris_params p{};
  std::vector<double> fw;
  int prec = IRIS_FP64;
  size_t esz = 16;  // bytes per stored complex value
  int device = 0;
  cudaStream_t st = nullptr;
  iris::Geo g{};
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
  iris::SrcArgs src{};
  dim3 tf_blk, tf_grd;
  // DFT
  int nboxes = 1;
  iris::FaceMap fm[2][3];
  long P = 0;
  int K = 0, nslot = 0;
  std::vector<iris::Seg> segs;
  long max_seg = 0;
  iris::Seg* d_segs = nullptr;
  void* S = nullptr;
  int* d_tk = nullptr;
  double* d_fw = nullptr;
  // accumulators [nof][P], 16 bytes a value: double2 in FP64 mode, the
  // double-float float4 (re_hi, im_hi, re_lo, im_lo) in FP32 mode
  void* fd = nullptr;
  // the accumulators hold no sum yet (no block committed since they were
  // allocated): their memory is left unwritten, the tensor-core commit
  // writes its first block without reading them and the tensor-core flux
  // read takes them as zeros; every other reader zeroes them first
  // (fd_materialise)
  bool fd_zero = false;
  float2* d_wt = nullptr;
  double2* d_wt64 = nullptr;  // FP64 mode twiddles of one block
  bool dft_tc = false;     // FP32 block accumulation on the tensor cores
  float* d_wtc = nullptr;  // its B operands (k_twiddle_tc)
  int ws_blocks = 0;       // CTAs of its persistent launches (one per SM)
  // flux faces as uploaded to d_faces (6 per set), and the flux partials of
  // the tensor-core flux read (4 per tile of the largest set, x nof)
  std::vector<iris::FluxFace> flux_faces;
  double* d_part = nullptr;
  iris::FluxFace* d_faces = nullptr;
  double* d_J = nullptr;
  double* h_J = nullptr;
  // batch member: no DFT buffers of its own; z-plane DFT only on request
  bool member = false;
  bool dft_z_only = false;
  std::vector<iris::FluxFace> host_faces;
  // fused E+H stepping (FP32): second field buffers and D, per-step TF/SF table
  bool fused = false;
  void* e2 = nullptr;
  void* h2 = nullptr;
  void* pml_d2[2] = {nullptr, nullptr};
  // z chunks (first, last plane) of its two launches: [0] the planes outside
  // the UPML slabs, [1] the slabs
  std::vector<int> fzr[2];
  dim3 fblk, fgrd;
  bool fz_i32 = false;  // the fused pass's offsets fit int (3 x comp < 2^31)
  // the slab launch runs on st2, concurrently with the interior launch (they
  // write disjoint planes and read only the old state): fork / join events
  cudaStream_t st2 = nullptr;
  cudaEvent_t fz_fork = nullptr, fz_join = nullptr;
  // CUDA graph of one DFT block of steps (iris_params.graph): d_it holds the
  // step base the captured kernels add to their offsets, dev_it its value
  cudaGraphExec_t gexec = nullptr;
  int* d_it = nullptr;
  int dev_it = -1;
  // persistent whole-step kernel (small grids): CTAs and threads per CTA of
  // its cooperative launch and its grid-barrier words
  bool persist = false;
  int persist_blocks = 0, persist_threads = 0;
  void* d_bar = nullptr;
  // its TF/SF corrections (vE, vH) per [step of a span][ix], up to tfv_cap steps
  iris::TfsfVal* d_tfv = nullptr;
  int tfv_cap = 0;
  long* d_sidx = nullptr;  // its DFT sample points: storage index * 8 + field
  // staging buffer of the complex(8) field transfers (allocated on first use)
  void* d_stage = nullptr;
  size_t stage_bytes = 0;
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

namespace iris {

// An NVTX range over one ABI call (visible in Nsight timelines; NVTX costs a
// branch when no tool is attached).
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange&) = delete;
  NvtxRange& operator=(const NvtxRange&) = delete;
};

// Brackets one kernel launch (or the fused pass's two concurrent launches)
// with a pair of events when timing is on.
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

// Engine lifetime.  member: a batch member (no DFT buffers of its own);
// z_only: DFT points on the z faces only; packed: rows of nx+2 cells back to
// back (no 128-byte alignment of x = 1), for cells whose rows are short.
int create_engine(const iris_params* pin, const double* fw, bool member, bool z_only, iris_engine** out,
                  bool packed = false);
void free_engine(iris_engine* E);
// DFT buffers for E->P sample points and nfaces flux faces.
int alloc_dft(iris_engine* E, const FluxFace* faces, int nfaces);
// Accumulate the sample ring into fdata (one block kernel pass).
void dft_flush(iris_engine* E);
// Zero the accumulators in memory if they hold no sum yet (fd_zero), before
// a kernel or copy that reads them as they lie.
int fd_materialise(iris_engine* E);
// Flux of face set `set` (6 FluxFace from d_faces + 6 set) into J[6][nof].
int read_flux(iris_engine* E, int set, double* J);
// One step (the fused pass or the split E and H passes, as the engine
// steps, then TF/SF), with the DFT sample of step it when dft is set and the
// step is sampled.
void one_step(iris_engine* E, int it, bool dft);

// Bounds-check records of the batch and adjoint modules (read and cleared;
// 0 in the ordinary build).
unsigned long long bc_take_batch();
unsigned long long bc_take_adjoint();

// CUDA graph of one DFT block of steps.
bool graph_ready(const iris_engine* E, int it, int left);
void graph_reset(iris_engine* E);
int graph_block(iris_engine* E, int it, const std::function<void()>& record);

}  // namespace iris
