// GB300 (sm_103a) FDTD engine, batched form.

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "iris_engine.h"
#include "iris_fused.cuh"

using namespace iris;

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

unsigned long long bc_take_batch() { return bc_take_module(); }

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
struct FItem {
  int cell, bx, by, z0, z1, pad;  // column tile (bx, by) of cell, planes z0..z1
};

// Work-list shapes the autotuner chooses from: x * y * z blocks of cells,
// (FLAT) 256 consecutive cells of one plane in row-major order, which keeps
// every lane busy whatever the cell's nx (FLAT: register-capped for five
// resident blocks per SM; FLAT + 1: uncapped), and (FUSED, FP32 only) the
// fused E+H pass over 32 x 16 column tiles and z chunks of every cell.
constexpr int NTILES = 8, FLAT = 5, FUSED = 7;
constexpr int TILES[NTILES][3] = {{32, 8, 1}, {32, 4, 2}, {64, 4, 1}, {16, 16, 1},
                                  {32, 2, 4}, {256, 1, 1}, {256, 1, 1}, {FZ_X, FZ_Y, 1}};
constexpr int FB_CHUNK = 64;  // planes per FUSED item outside the UPML slabs
static_assert(NTILES == IRIS_BATCH_NTILES, "the ABI's candidate count");

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

// The fused E+H pass over FUSED items: one tile column of one cell per
// item, the cell's FusedArgs (for the current buffer parity) copied to
// shared memory when the item's cell changes.  UPML as in k_fused: items
// outside the slabs with the kernel compiled without slab code.  CEPS: the
// batch holds a complex material somewhere; each item still picks the
// column for its own cell's material (a real one has no complex table).
template <bool CEPS, bool UPML>
__global__ void __launch_bounds__(FZ_X* FZ_Y, 2) k_batch_fused(const FusedArgs* __restrict__ args,
                                                             const FItem* __restrict__ items, long nitems) {
  __shared__ FusedSmem S;
  __shared__ __align__(16) FusedArgs sa;
  __shared__ int scell;
  extern __shared__ __align__(16) unsigned char fz_dyn[];
  FusedUpml& U = *reinterpret_cast<FusedUpml*>(fz_dyn);  // UPML = true only
  const int tid = threadIdx.y * FZ_X + threadIdx.x;
  if (tid == 0) scell = -1;
  for (long k = blockIdx.x; k < nitems; k += gridDim.x) {
    const FItem it = items[k];
    __syncthreads();  // the previous item's last reads of S and sa are done
    if (it.cell != scell) {
      const int* src = (const int*)(args + it.cell);
      for (int i = tid; i < (int)(sizeof(FusedArgs) / 4); i += FZ_X * FZ_Y) ((int*)&sa)[i] = src[i];
      __syncthreads();
      if (tid == 0) scell = it.cell;
    }
    // CEPS: some cell of the batch has a complex material; cells with a real
    // one (eps_c null) still take the real-material column
    if (CEPS && sa.f.eps_c) fused_column<true, UPML>(sa, S, U, it.bx, it.by, it.z0, it.z1);
    else fused_column<false, UPML>(sa, S, U, it.bx, it.by, it.z0, it.z1);
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
                                                      int t, const int* tp, long np) {
  if (blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0) tk[islot] = tp ? *tp + t : t;
  const BSeg b = segs[blockIdx.y];
  if (blockIdx.x * (unsigned)GATHER_BLOCK >= (unsigned)b.s.nu * (unsigned)b.s.nv) return;
  const FieldArgs<T>& a = args[b.cell];
  const typename V2<T>::t* src = b.s.field < 3 ? a.e + b.s.field * a.g.comp : a.h + (b.s.field - 3) * a.g.comp;
  gather_run<T>(b.s, src, slot, a.g.comp, np);
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
  void* d_args = nullptr;  // FieldArgs<T>[2][n]: the cells' current fields at buffer parity 0, 1
  // FUSED: the members' second field buffers exist; parity: which buffer set
  // holds the current fields (0 = the members' first buffers); d_fargs:
  // FusedArgs[2][n] (old fields at parity q, new ones in the other set)
  bool second = false;
  int parity = 0;
  void* d_fargs = nullptr;
  FItem* d_fitems = nullptr;
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

// Swaps a member's field, second-field and D buffers.
void swap_sets(iris_engine* E) {
  std::swap(E->e, E->e2);
  std::swap(E->h, E->h2);
  for (int s = 0; s < 2; ++s) std::swap(E->pml_d[s], E->pml_d2[s]);
}

// The cells' kernel arguments for both buffer parities.  A member's own
// pointers always name its current fields (parity B->parity).
int batch_upload_args(iris_batch* B) {
  const size_t sz = B->prec == IRIS_FP64 ? sizeof(FieldArgs<double>) : sizeof(FieldArgs<float>);
  std::vector<unsigned char> h(2 * sz * B->n);
  std::vector<FusedArgs> fa(B->second ? 2 * B->n : 0);
  for (int q = 0; q < 2; ++q)
    for (int c = 0; c < B->n; ++c) {
      iris_engine* E = B->cells[c];
      const bool other = q != B->parity && B->second;
      if (other) swap_sets(E);  // view the set that is current at parity q
      if (B->prec == IRIS_FP64) {
        FieldArgs<double> a = field_args<double>(E);
        std::memcpy(h.data() + sz * ((size_t)q * B->n + c), &a, sz);
      } else {
        FieldArgs<float> a = field_args<float>(E);
        std::memcpy(h.data() + sz * ((size_t)q * B->n + c), &a, sz);
        if (B->second) {
          FusedArgs& f = fa[(size_t)q * B->n + c];
          f = FusedArgs{};
          f.f = a;
          f.e_new = (float2*)E->e2;
          f.h_new = (float2*)E->h2;
          for (int s = 0; s < 2; ++s) f.d_new[s] = (float2*)E->pml_d2[s];
        }
      }
      if (other) swap_sets(E);
    }
  if (!B->d_args) CK(cudaMalloc(&B->d_args, h.size()));
  CK(cudaMemcpy(B->d_args, h.data(), h.size(), cudaMemcpyHostToDevice));
  if (B->second) {
    if (!B->d_fargs) CK(cudaMalloc(&B->d_fargs, sizeof(FusedArgs) * fa.size()));
    CK(cudaMemcpy(B->d_fargs, fa.data(), sizeof(FusedArgs) * fa.size(), cudaMemcpyHostToDevice));
  }
  return IRIS_OK;
}

// Frees the members' second buffer sets (tuning only: every set holds the
// zero state then, so the first one can be made current without a copy).
int batch_drop_second(iris_batch* B) {
  CK(cudaStreamSynchronize(B->master->st));
  if (B->parity) {
    for (iris_engine* E : B->cells) swap_sets(E);
    B->parity = 0;
  }
  bool any = B->second;
  for (iris_engine* E : B->cells) {
    void* ptrs[] = {E->e2, E->h2, E->pml_d2[0], E->pml_d2[1]};
    for (void* q : ptrs)
      if (q) {
        cudaFree(q);
        any = true;
      }
    E->e2 = E->h2 = nullptr;
    E->pml_d2[0] = E->pml_d2[1] = nullptr;
  }
  B->second = false;
  return any ? batch_upload_args(B) : IRIS_OK;
}

// The members' second field buffers and D (zero), for the FUSED work list.
int batch_second_buffers(iris_batch* B) {
  if (B->second) return IRIS_OK;
  for (iris_engine* E : B->cells) {
    const size_t fbytes = (size_t)3 * E->g.comp * E->esz;
    if (!E->e2) CK(cudaMalloc(&E->e2, fbytes));
    if (!E->h2) CK(cudaMalloc(&E->h2, fbytes));
    CK(cudaMemsetAsync(E->e2, 0, fbytes, B->master->st));
    CK(cudaMemsetAsync(E->h2, 0, fbytes, B->master->st));
    for (int s = 0; s < 2; ++s) {
      const size_t b = (size_t)3 * E->pcomp[s] * E->esz;
      if (!E->pml_d2[s]) CK(cudaMalloc(&E->pml_d2[s], std::max<size_t>(b, 16)));
      CK(cudaMemsetAsync(E->pml_d2[s], 0, std::max<size_t>(b, 16), B->master->st));
    }
  }
  B->second = true;
  return batch_upload_args(B);
}

// FUSED items: every cell's planes outside its UPML slabs in chunks of
// FB_CHUNK (stopping at pmlzf-2, as the single-engine launch does) first,
// then its two slabs each with the plane next to it; within a chunk, tile
// rows of the cell in order.
int batch_build_fused_items(iris_batch* B) {
  std::vector<FItem> in, slab;
  for (int c = 0; c < B->n; ++c) {
    const iris_params& p = B->cells[c]->p;
    const int tx = (p.nx + FZ_OX - 1) / FZ_OX, ty = (p.ny + FZ_OY - 1) / FZ_OY;
    auto add = [&](std::vector<FItem>& v, int za, int zb, int len) {
      for (int z = za; z <= zb; z += len)
        for (int by = 0; by < ty; ++by)
          for (int bx = 0; bx < tx; ++bx) v.push_back(FItem{c, bx, by, z, std::min(z + len - 1, zb), 0});
    };
    const int ia = p.pmlzi + 1, ib = p.pmlzf - 2;
    if (ib >= ia) {
      add(in, ia, ib, FB_CHUNK);
      add(slab, 1, ia - 1, p.nz);
      add(slab, ib + 1, p.nz, p.nz);
    } else {
      add(slab, 1, p.nz, p.nz);
    }
  }
  B->nitems_in = (long)in.size();
  in.insert(in.end(), slab.begin(), slab.end());
  for (const void* kf : {(const void*)k_batch_fused<false, true>, (const void*)k_batch_fused<true, true>})
    CK(cudaFuncSetAttribute(kf, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)FZ_UPML_SMEM));
  graph_reset(B->master);
  if (B->d_fitems) cudaFree(B->d_fitems);
  B->d_fitems = nullptr;
  CK(cudaMalloc(&B->d_fitems, sizeof(FItem) * std::max<size_t>(1, in.size())));
  CK(cudaMemcpy(B->d_fitems, in.data(), sizeof(FItem) * in.size(), cudaMemcpyHostToDevice));
  B->nitems = (long)in.size();
  B->tile = FUSED;
  B->master->fused = true;  // graphs of an even number of steps only (the buffer sets alternate)
  return IRIS_OK;
}

int batch_build_items(iris_batch* B, int tile) {
  if (tile == FUSED) {
    if (B->prec != IRIS_FP32) return fail(IRIS_EINVAL, "the fused work list is FP32 only");
    int rc = batch_second_buffers(B);
    if (rc) return rc;
    return batch_build_fused_items(B);
  }
  B->master->fused = false;
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

// The cells' FieldArgs<T> for the current buffer parity.
template <typename T> const FieldArgs<T>* cur_args(const iris_batch* B) {
  return (const FieldArgs<T>*)B->d_args + (size_t)B->parity * B->n;
}

template <typename T, int TX, int TY, int TZ> void launch_batch_eh(iris_batch* B, bool e) {
  iris_engine* M = B->master;
  const dim3 blk(TX, TY, TZ);
  const FieldArgs<T>* args = cur_args<T>(B);
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
  const FieldArgs<T>* args = cur_args<T>(B);
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

// One fused E+H pass of every cell (FUSED work list, FP32): the items
// outside the slabs, then the slab items; the buffer sets then swap.
template <bool CEPS> void launch_batch_fused(iris_batch* B) {
  iris_engine* M = B->master;
  const FusedArgs* args = (const FusedArgs*)B->d_fargs + (size_t)B->parity * B->n;
  for (int part = 0; part < 2; ++part) {
    const long n = part == 0 ? B->nitems_in : B->nitems - B->nitems_in;
    if (n <= 0) continue;
    const FItem* items = B->d_fitems + (part == 0 ? 0 : B->nitems_in);
    const void* kern = part == 0 ? (const void*)k_batch_fused<CEPS, false> : (const void*)k_batch_fused<CEPS, true>;
    const size_t dyn = part == 0 ? 0 : FZ_UPML_SMEM;
    static int per[2] = {0, 0};
    if (!per[part]) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per[part], kern, FZ_X * FZ_Y, dyn);
    int nsm = 0;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, B->device);
    const unsigned g = (unsigned)std::min<long>(n, (long)nsm * std::max(1, per[part]));
    KTimer tm(M, IRIS_KC_FUSED);
    if (part == 0) k_batch_fused<CEPS, false><<<g, dim3(FZ_X, FZ_Y), 0, M->st>>>(args, items, n);
    else k_batch_fused<CEPS, true><<<g, dim3(FZ_X, FZ_Y), FZ_UPML_SMEM, M->st>>>(args, items, n);
  }
  B->parity ^= 1;
  for (iris_engine* E : B->cells) swap_sets(E);
}

void batch_fused(iris_batch* B) {
  bool cplx = false;
  for (const iris_engine* E : B->cells) cplx |= E->eps_complex;
  if (cplx) launch_batch_fused<true>(B);
  else launch_batch_fused<false>(B);
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
  if (B->tile == FUSED) {
    batch_fused(B);
  } else {
    batch_eh<T>(B, true);
    batch_eh<T>(B, false);
  }
  const FieldArgs<T>* args = cur_args<T>(B);  // after the fused pass: the new set
  if (B->ntitems) {
    KTimer tm(M, IRIS_KC_TFSF);
    const long g = std::min<long>(B->ntitems, 152L * 16);
    k_batch_tfsf<T><<<(unsigned)g, 64, 0, M->st>>>(args, B->d_src, B->d_titems, B->ntitems, it, itp);
  }
  if (sampled) {
    {
      KTimer tm(M, IRIS_KC_GATHER);
      V* slot = (V*)M->S + (long)M->nslot * M->P;
      dim3 grid((unsigned)((B->max_seg + GATHER_BLOCK - 1) / GATHER_BLOCK), (unsigned)B->nbsegs);
      k_batch_gather<T><<<grid, 256, 0, M->st>>>(args, B->d_bsegs, slot, M->d_tk, M->nslot, it + 1 - p.to_fourier,
                                                 itp, M->P);
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
  void* ptrs[] = {B->d_args, B->d_src, B->d_items, B->d_titems, B->d_bsegs, B->d_fargs, B->d_fitems};
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
  iris::NvtxRange nvtx_("iris_batch_create");
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

int iris_batch_material_pattern(iris_batch* B, int cell, unsigned long long seed, double fill, double eps_in,
                                double eps_out) {
  clear_error();
  if (!B || cell < 0 || cell >= B->n) return fail(IRIS_EINVAL, "bad argument");
  CK(cudaSetDevice(B->device));
  CK(cudaStreamSynchronize(B->master->st));
  int rc = iris_material_pattern(B->cells[cell], seed, fill, eps_in, eps_out);
  if (rc) return rc;
  return batch_upload_args(B);  // the material pointer has changed
}

int iris_batch_step(iris_batch* B, int it0, int nsteps) {
  iris::NvtxRange nvtx_("iris_batch_step");
  clear_error();
  if (!B || nsteps < 0) return fail(IRIS_EINVAL, "bad argument");
  CK(cudaSetDevice(B->device));
  return B->prec == IRIS_FP64 ? batch_step_t<double>(B, it0, nsteps) : batch_step_t<float>(B, it0, nsteps);
}

int iris_batch_flux(iris_batch* B, int cell, double* J) {
  iris::NvtxRange nvtx_("iris_batch_flux");
  clear_error();
  if (!B || !J || cell < 0 || cell >= B->n) return fail(IRIS_EINVAL, "bad argument");
  CK(cudaSetDevice(B->device));
  return read_flux(B->master, cell, J);
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

namespace {

// The autotuner's picks by size class: in the process, and in the file named
// by IRIS_TUNE_CACHE when set (lines "<class> <tile>", read once, appended to).
std::mutex g_tune_mu;
std::map<std::string, int> g_tune;
bool g_tune_loaded = false;

// Size class of a batch: the device, the precision, a complex material, and
// the binary orders of magnitude of the cell count, the total grid cells and
// the mean nx, ny and nz (the work lists' efficiency follows row lengths and
// the amount of work).
std::string size_class(const iris_batch* B) {
  cudaDeviceProp prop{};
  cudaGetDeviceProperties(&prop, B->device);
  double sx = 0, sy = 0, sz = 0, tot = 0;
  bool cplx = false;
  for (const iris_engine* E : B->cells) {
    sx += E->p.nx;
    sy += E->p.ny;
    sz += E->p.nz;
    tot += (double)E->p.nx * E->p.ny * E->p.nz;
    cplx |= E->eps_complex;
  }
  const double n = std::max(1, B->n);
  auto lg = [](double v) { return (int)std::floor(std::log2(std::max(1.0, v))); };
  std::string name(prop.name);
  for (char& c : name)
    if (c == ' ') c = '_';
  return name + "|sm" + std::to_string(prop.multiProcessorCount) + (B->prec == IRIS_FP64 ? "|fp64" : "|fp32") +
         (cplx ? "|cplx" : "|real") + "|n" + std::to_string(lg(n)) + "|c" + std::to_string(lg(tot)) + "|x" +
         std::to_string(lg(sx / n)) + "|y" + std::to_string(lg(sy / n)) + "|z" + std::to_string(lg(sz / n));
}

void tune_cache_load() {
  if (g_tune_loaded) return;
  g_tune_loaded = true;
  const char* path = std::getenv("IRIS_TUNE_CACHE");
  if (!path || !*path) return;
  FILE* f = std::fopen(path, "r");
  if (!f) return;
  char key[256];
  int t;
  while (std::fscanf(f, "%255s %d", key, &t) == 2)
    if (t >= 0 && t < NTILES) g_tune[key] = t;
  std::fclose(f);
}

void tune_cache_store(const std::string& key, int t) {
  g_tune[key] = t;
  const char* path = std::getenv("IRIS_TUNE_CACHE");
  if (!path || !*path) return;
  if (FILE* f = std::fopen(path, "a")) {
    std::fprintf(f, "%s %d\n", key.c_str(), t);
    std::fclose(f);
  }
}

}  // namespace

int iris_batch_autotune(iris_batch* B, int reps, int* best, int* cached) {
  clear_error();
  if (!B || reps < 1) return fail(IRIS_EINVAL, "bad argument");
  if (B->steps_taken) return fail(IRIS_EINVAL, "tune before the first step (it runs E and H passes on the state)");
  CK(cudaSetDevice(B->device));
  const std::string key = size_class(B);
  int t = -1;
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    tune_cache_load();
    auto it = g_tune.find(key);
    if (it != g_tune.end() && !(it->second == FUSED && B->prec != IRIS_FP32)) t = it->second;
  }
  if (t >= 0) {
    int rc = iris_batch_set_tile(B, t);
    if (rc == IRIS_OK) {
      if (best) *best = t;
      if (cached) *cached = 1;
      return IRIS_OK;
    }
    clear_error();  // a pick this batch cannot take (memory): time the candidates
  }
  int rc = iris_batch_tune(B, reps, &t, nullptr);
  if (rc) return rc;
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    tune_cache_store(key, t);
  }
  if (best) *best = t;
  if (cached) *cached = 0;
  return IRIS_OK;
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
  // one E and one H pass, or one fused pass
  auto pass = [&] {
    if (B->tile == FUSED) batch_fused(B);
    else if (B->prec == IRIS_FP64) {
      batch_eh<double>(B, true);
      batch_eh<double>(B, false);
    } else {
      batch_eh<float>(B, true);
      batch_eh<float>(B, false);
    }
  };
  const int ntry = B->prec == IRIS_FP32 ? NTILES : FUSED;  // FUSED is FP32 only
  if (ms)
    for (int t = ntry; t < NTILES; ++t) ms[t] = -1.0;
  for (int t = 0; t < ntry; ++t) {
    int rc = batch_build_items(B, t);
    if (rc == IRIS_ENOMEM && t == FUSED) {
      // no room for the second buffer sets: not a candidate on this batch
      cudaGetLastError();
      clear_error();
      rc = batch_drop_second(B);
      if (rc) return rc;
      if (ms) ms[t] = -1.0;
      continue;
    }
    if (rc) return rc;
    // fields are still zero (both buffer sets), so the passes leave the state unchanged
    for (int r = 0; r < 2; ++r) pass();
    CK(cudaEventRecord(a, M->st));
    for (int r = 0; r < reps; ++r) pass();
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
  if (arg != FUSED) {
    int rc = batch_drop_second(B);
    if (rc) return rc;
  }
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
  info[6] = B->tile >= FLAT ? (B->nitems_in > 0) + (B->nitems > B->nitems_in) : 1;  // per E, H or fused pass
  info[7] = B->master->nslot;
  return IRIS_OK;
}

int iris_batch_dft_commit(iris_batch* B) {
  clear_error();
  if (!B) return fail(IRIS_EINVAL, "null batch");
  CK(cudaSetDevice(B->device));
  dft_flush(B->master);
  CK(cudaGetLastError());
  return IRIS_OK;
}

}  // extern "C"
