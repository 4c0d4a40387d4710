/*
 * iris_fdtd.h — C ABI of the GB300 FDTD time-stepping engine.
 *
 * A drop-in for the hot path of IrisFDTD-Academic (Fortran): the per-step
 * operators that driver() calls (code/driver.f90:338-451) and the run set-up
 * around them.  Every entry point below names the reference interface it
 * replaces.  Arrays cross the boundary as plain host pointers in the
 * reference's own layout; the engine owns all device memory.
 *
 * Conventions
 *   - Every call returns IRIS_OK (0) or a negative IRIS_E* code; no call
 *     aborts or exits (the reference's err() STOPs: code/files.f90:352-381).
 *   - Host buffers are borrowed for the duration of the call only.
 *   - One engine is driven by one host thread at a time; engines are
 *     independent and each runs on its own CUDA stream.
 *   - Time steps are numbered from 1 like the reference's `it`
 *     (code/driver.f90:338).
 *   - Field arrays in the reference layout are complex(8)
 *     (3, 0:nx+1, 0:ny+1, 0:nz+1), component fastest, passed as two double
 *     arrays (real parts, imaginary parts) of 3*(nx+2)*(ny+2)*(nz+2) values.
 */
#ifndef IRIS_FDTD_H
#define IRIS_FDTD_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes --------------------------------------------------- */
#define IRIS_OK 0
#define IRIS_EINVAL (-1)   /* bad argument or parameter combination          */
#define IRIS_ENOMEM (-2)   /* device or host allocation failed               */
#define IRIS_ECUDA (-3)    /* CUDA runtime error (message: iris_last_error)  */
#define IRIS_EPARSE (-4)   /* inputFDTD.dat could not be read                */
#define IRIS_EIO (-5)      /* output file could not be written               */
#define IRIS_ENAN (-6)     /* non-finite value detected in the flux          */
#define IRIS_ETIMEOUT (-7) /* a bounded device wait gave up                  */
#define IRIS_ENODEV (-8)   /* no CUDA device                                 */

/* ---- precision modes ------------------------------------------------ */
/* FP64 fields and DFT, operations in the reference's order (parity mode). */
#define IRIS_FP64 0
/* FP32 fields; TF/SF incident field in FP64; DFT partial sums over a block
 * of K samples in FP32 with FP64-exact twiddles, accumulated in FP64.     */
#define IRIS_FP32 1

/* ---- single operator groups (iris_apply) ----------------------------- */
#define IRIS_OP_E 1    /* e_fdtd + UPML_Array_e + bc_{x,y,z}max_bloch      */
#define IRIS_OP_H 2    /* h_fdtd + UPML_Array_h + bc_{x,y,z}min_bloch      */
#define IRIS_OP_TFSF 3 /* tfsf_gauss/tfsf_plane_wave + tfsf_update_{2D,3D} */
#define IRIS_OP_DFT 4  /* scattering_fourier for every box, arg = time idx */
/* Check of the bounded device waits: one CTA arms an mbarrier for bytes
 * that are never sent, waits on it with the limit the streamed passes use
 * divided by 2^arg (arg 0..30), gives up, records it like a real give-up
 * and returns.  iris_apply then returns IRIS_ETIMEOUT; the engine and its
 * CUDA context stay usable.  No memory is touched but the engine's
 * error word.                                                          */
#define IRIS_OP_WAIT_CHECK 5
/* The same for the persistent kernel's grid barrier: a cooperative launch of
 * two CTAs in which one never arrives; the other waits with the persistent
 * kernel's limit divided by 2^arg (arg 0..30), gives up and records it.
 * IRIS_ETIMEOUT; the engine stays usable.  Engines stepping with the
 * persistent kernel only.                                              */
#define IRIS_OP_BARRIER_CHECK 6

/* ---- field selectors (iris_get_field / iris_set_field) --------------- */
#define IRIS_E 0
#define IRIS_H 1

/*
 * Run parameters: the `module parameters` state after setparam()
 * (code/parameters.f90:25-261, code/files.f90:39-344), in atomic units.
 */
typedef struct iris_params {
  /* 'Mesh options' */
  int i_pol;          /* 1: E//y, 2: E//x                                  */
  int nx, ny, nz;     /* ixmax, iymax, izmax                               */
  int pmlzi, pmlzf;   /* UPML slabs z in [1,pmlzi] and [pmlzf,nz]          */
  int npml;           /* UPML grading exponent nPML (the reference fixes 2) */
  int pml_taflove;    /* value read from the nPML line (unused)            */
  double q_nm, Q;     /* cell size in nm, and in bohr                      */
  double cfl, dt;     /* CFL number; time step in a.u.                     */
  double wzpml;       /* UPML strength after the f_abohr/Q rescaling       */
  /* 'Job options' */
  int no_downloads;   /* output interval in steps: int(texit/no_downloads) */
  int output_time_step;
  int texit;          /* number of time steps                              */
  double texit_fs;
  int hi, hf;         /* structure z-range [hi, hf]                        */
  int sdl_plane_on[3];
  /* 'Dielectric constants' */
  double eps1, eps3;  /* cover and substrate                               */
  double eps_bbox_re, eps_bbox_im;
  /* 'Fourier transformation options' */
  int box1[6];        /* sxi, sxf, syi, syf, szi, szf                      */
  int box2[6];        /* mxi, mxf, myi, myf, mzi, mzf                      */
  int nof;            /* number of frequencies                             */
  double dlamda, lno; /* wavelength step and first wavelength in nm        */
  int to_fourier, sample_fourier;
  /* 'Source options' */
  int plane_wave;     /* 1: Gaussian pulse, 0: CW with ramps               */
  int tfsf_zi, tfsf_zf; /* iz_min and iz_max (= tfsf_zi + 5)               */
  int cosine;         /* 1: real-valued source                             */
  double epump;       /* amplitude in a.u. (Epump and Eoxy)                */
  double wlpump;      /* wavelength in nm                                  */
  double pump_dt;     /* pulse duration in a.u.                            */
  double def_pulse;
  double gpump, zopump; /* pulse width (cells) and origin                  */
  double tincr, tdecay; /* CW switch-on / switch-off times in a.u.         */
  double gap;         /* GAP, never set by the reference (0)               */
  double ratio_angle; /* 1: normal incidence                               */
  /* 'Slit Array' */
  int dh, dx, aix, afx;
  /* constants as the reference evaluates them (code/physconst.f90:31-53) */
  double pi, c0, eps0, mu0, f_abohr, uat, f_e, pmlalfa;
  /* Bloch phases per period: complex akx, aky, akz (code/parameters.f90:85,
   * never assigned by the reference, so 0 there)                          */
  double akx_re, akx_im, aky_re, aky_im, akz_re, akz_im;
  int system_model;   /* never assigned by the reference: 0                */
  /* engine options (not part of the reference) */
  int precision;      /* IRIS_FP64 or IRIS_FP32                            */
  int dft_block;      /* samples buffered per DFT accumulation; 0: default
                       * (FP32 512, FP64 32; at most 512 / 256, halved
                       * while the ring would exceed half the memory left
                       * after the accumulators)                          */
  int device;         /* CUDA device ordinal                               */
  int stencil;        /* IRIS_STENCIL_*: how E and H are stepped           */
  int dft_faces;      /* IRIS_DFT_ALL or IRIS_DFT_Z                        */
  int graph;          /* 1: step whole DFT blocks (every step sampled) by
                         replaying one captured CUDA graph; results are
                         identical to launch-by-launch stepping            */
  int dft_kernel;     /* IRIS_DFT_KERNEL_*: FP32 DFT block accumulation    */
} iris_params;

/* ---- FP32 DFT block kernels (iris_params.dft_kernel) ------------------ */
#define IRIS_DFT_KERNEL_AUTO 0   /* the engine's choice (tensor cores)      */
#define IRIS_DFT_KERNEL_CUDA 1   /* FP32 FMA on the CUDA cores              */
/* tcgen05 tensor cores, TF32 operands split hi + lo (three MMAs per product,
 * FP32-level accuracy), FP32 partial sums in TMEM, FP64 accumulators      */
#define IRIS_DFT_KERNEL_TENSOR 2

/* ---- DFT faces (iris_params.dft_faces) -------------------------------- */
/* every face pair scattering_fourier accumulates (the reference)          */
#define IRIS_DFT_ALL 0
/* only the two z planes (reflection and transmission, all T/R needs)      */
#define IRIS_DFT_Z 1

/* ---- stencil variants (iris_params.stencil) -------------------------- */
/* default: the persistent kernel on small grids, else the fused pass in
 * IRIS_FP32 (the faster variant on GB300; the split passes instead on
 * grids whose x-y plane would leave more than half of the fused pass's
 * 32 x 16 tile threads idle, e.g. 4 cells in y) and the split passes in
 * IRIS_FP64                                                               */
#define IRIS_STENCIL_DEFAULT 0
/* separate in-place E and H passes (18 complex values per cell per step)  */
#define IRIS_STENCIL_SPLIT 1
/* one fused E+H pass over double-buffered fields (12 values per cell, twice
 * the field memory); IRIS_FP32 only                                       */
#define IRIS_STENCIL_FUSED 2
/* the split passes with each plane staged in shared memory by bulk (TMA)
 * copies, z-marching tiles; IRIS_FP32 with a real material (a complex
 * material steps with the split passes)                                   */
#define IRIS_STENCIL_STREAM 3
/* small grids: one cooperative launch runs a span of whole steps (E, H,
 * TF/SF, DFT sample) with grid-wide barriers between the passes; the split
 * passes' arithmetic, so the same results bit for bit.  The default for
 * IRIS_FP64 grids of at most IRIS_PERSISTENT_MAX_CELLS cells and IRIS_FP32
 * grids of at most IRIS_PERSISTENT_MAX_CELLS_FP32 cells (up to those sizes
 * it steps faster than the split passes, and the split passes than the
 * fused pass); asked for explicitly, grids of fewer than
 * 2^31 / 3 cells on a device with cooperative launches (else iris_create
 * returns IRIS_EINVAL)                                                    */
#define IRIS_STENCIL_PERSISTENT 4
#define IRIS_PERSISTENT_MAX_CELLS 1048576
#define IRIS_PERSISTENT_MAX_CELLS_FP32 8388608

typedef struct iris_engine iris_engine;

/* Human-readable text of a status code / of the last error on this thread. */
const char* iris_strerror(int status);
const char* iris_last_error(void);

/*
 * Read inputFDTD.dat and fill *out; replaces setparam()
 * (code/files.f90:39-344) with the reference's section scanning, list-
 * directed reads, unit conversions and truncations.  fw receives the nof
 * angular frequencies (code/files.f90:216-220) when fw_cap >= nof.
 * desc (optional) receives the first line of the file (code/main.f90:111).
 * single_literals: 1 evaluates unsuffixed literals as REAL(4), as standard
 * Fortran does; 0 evaluates them in double.
 */
int iris_setparam(const char* input_path, int single_literals, iris_params* out,
                  double* fw, int fw_cap, char* desc, int desc_cap);

/* The constants of code/physconst.f90 into p (called by iris_setparam). */
void iris_physconsts(iris_params* p, int single_literals);

/* Angular frequencies fw(1:nof) from lno/dlamda, code/files.f90:216-220. */
int iris_frequencies(const iris_params* p, double* fw, int fw_cap);

/*
 * Allocate and initialise one run: fields e,h = 0 (code/main.f90:166-170),
 * the UPML slabs and set_sz() profiles (code/driver.f90:177-200,
 * code/boundary_II.f90:224-276), the DFT sample tables and accumulators of
 * both boxes (code/driver.f90:205-286, code/dataprocess.f90:793-903), the
 * TF/SF scratch (code/driver.f90:310-331) and the material of
 * set_emconstants() + slit() (code/mesh.f90:57-109).
 */
int iris_create(const iris_params* p, const double* fw, iris_engine** out);
void iris_destroy(iris_engine* eng);

/*
 * Replace the inverse permittivity eps_inv(1,1,0:nx+1,0:ny+1,hi-1:hf+1)
 * (code/mesh.f90:102-106), x fastest, as re/im arrays of
 * (nx+2)*(ny+2)*(hf-hi+3) values (im may be NULL: real material).
 * This is the hook the reference points users to for their own structures
 * (modify slit(), code/mesh.f90:65-66).
 */
int iris_set_material(iris_engine* eng, const double* eps_inv_re, const double* eps_inv_im);

/*
 * Material generators: the structure's eps_inv over planes hi..hf built on
 * the device instead of uploaded (the geometry front-end; slit(),
 * code/mesh.f90:57-69, is the reference's only generator).  Each replaces
 * the whole structure material like iris_set_material, as a real material
 * over the background 1/eps_bbox (eps_bbox must be real).
 *   spheres: n rows (cx, cy, cz, r, eps), in order, later rows win; a cell
 *     takes 1/eps where ((z-cz)^2 + (y-cy)^2) + (x-cx)^2 <= r^2, over the
 *     sphere's bounding box clipped to [hi, hf] in z and to nx, ny cells from
 *     floor(c - r) in x, y, taken modulo the period; ghost rows and columns
 *     hold their periodic images.
 *   pattern: 1/eps_in where the i-th draw of a SplitMix64 stream started at
 *     seed is below fill, else 1/eps_out; i = ((z-hi)*ny + y-1)*nx + x-1;
 *     ghosts as above.
 *   design: 1/(emin + (emax-emin)*u_i) over region {x0, x1, y0, y1} (all
 *     planes hi..hf), u_i the i-th draw, i in the region's own (z, y, x)
 *     order; 1/eps_bbox elsewhere, ghosts included.
 * The draws: state = seed + (i+1)*0x9E3779B97F4A7C15, SplitMix64's
 * finaliser, top 53 bits times 2^-53.
 */
int iris_material_spheres(iris_engine* eng, int n, const double* spheres);
int iris_material_pattern(iris_engine* eng, unsigned long long seed, double fill, double eps_in, double eps_out);
int iris_material_design(iris_engine* eng, unsigned long long seed, const int region[4], double emin, double emax);
/* The stored material, planes hi..hf: re/im arrays of (hf-hi+1)*(ny+2)*(nx+2)
 * values, x fastest (im is 0 for a real material). */
int iris_get_material(iris_engine* eng, double* re, double* im);

/*
 * Advance the fields by nsteps steps, it = it0 .. it0+nsteps-1: the body of
 * the time loop, code/driver.f90:356-451, in the reference's order:
 * E (all regions), UPML-E, Bloch max ghosts, H, UPML-H, Bloch min ghosts,
 * TF/SF source, then the DFT sample of E and H when it >= to_fourier and
 * mod(it, sample_fourier) == 0.  Asynchronous on the engine's stream.
 */
int iris_step(iris_engine* eng, int it0, int nsteps);

/* Wait for the engine's stream; reports any deferred CUDA error. */
int iris_sync(iris_engine* eng);

/*
 * Poynting flux per face of box 1 or 2 (box = 0 or 1), J[6][nof], face-
 * major: the Jabs array of scattering_fourier_out
 * (code/dataprocess.f90:243-277), eps0*Q/(2 dt) included.  Returns
 * IRIS_ENAN if any value is not finite.  Every sample taken so far counts;
 * in IRIS_FP32 mode (tensor-core DFT) the samples still buffered are added
 * on the fly and stay buffered, so a flux read changes no state.
 */
int iris_flux(iris_engine* eng, int box, double* J);

/*
 * Accumulate the DFT samples still buffered into fdata now (the engine
 * otherwise does so when its buffer of dft_block samples is full, and
 * before iris_get_fdata).  The running sum of scattering_fourier
 * (code/dataprocess.f90:143-147) is the same either way.
 */
int iris_dft_commit(iris_engine* eng);

/*
 * Append one output block to <box>_scatt1..6.dat and <box>_scatt.dat in
 * dir, as scattering_fourier_out does (code/dataprocess.f90:279-299).
 */
int iris_write_scatt(const char* dir, int box, int it, int nof, const double* J);

/* Field access in the reference layout (see top of file). */
int iris_get_field(iris_engine* eng, int which, double* re, double* im);
int iris_set_field(iris_engine* eng, int which, const double* re, const double* im);

/*
 * The same in the reference's own storage: c is the complex(8) array
 * e(3, 0:nx+1, 0:ny+1, 0:nz+1) or h(...) of code/main.f90:166-167 (and of
 * driver()'s e_cur, h_cur, code/driver.f90:301-302) as interleaved
 * (re, im) doubles (C99 double _Complex, Fortran complex(c_double_complex)),
 * 6*(nx+2)*(ny+2)*(nz+2) doubles.  A Fortran host passes its arrays
 * directly: the engine converts on the device, a few z planes at a time
 * through a staging buffer of at most 64 MB (or one plane), so no host copy
 * of the field is made.
 */
int iris_get_field_c(iris_engine* eng, int which, double* c);
int iris_set_field_c(iris_engine* eng, int which, const double* c);

/*
 * UPML auxiliaries d (which = 0) or b (which = 1) of slab 0 (z in
 * [1,pmlzi]) or slab 1 (z in [pmlzf,nz]) in the reference layout
 * (3,1:nx,1:ny,slab) (code/driver.f90:177-188), re/im arrays.
 */
int iris_get_pml(iris_engine* eng, int which, int slab, double* re, double* im);
int iris_set_pml(iris_engine* eng, int which, int slab, const double* re, const double* im);
/* The same as complex(8) arrays (3,1:nx,1:ny,slab planes), interleaved
 * (re, im) doubles, converted on the device like iris_get_field_c. */
int iris_get_pml_c(iris_engine* eng, int which, int slab, double* c);
int iris_set_pml_c(iris_engine* eng, int which, int slab, const double* c);

/*
 * One plane of E or H extracted on the device, for the SDL snapshots of
 * SDL_output (code/sdl.f90:68-234): axis 1, 2, 3 = the plane x, y, z = index;
 * the two in-plane coordinates run over [lo1, hi1] x [lo2, hi2] (y, z for
 * axis 1; x, z for axis 2; x, y for axis 3), ghost cells 0 and n+1 allowed.
 * re/im receive 3 * n1 * n2 values, component fastest, then the first
 * in-plane coordinate.
 */
int iris_get_plane(iris_engine* eng, int which, int axis, int index, int lo1, int hi1, int lo2, int hi2,
                   double* re, double* im);

/*
 * DFT accumulator emg(j)%fdata(i_pts, iw) of box (0/1) and face pair
 * j (1..3) in the reference order, i_pts fastest
 * (code/dataprocess.f90:109-209); *npts receives the point count.
 * Call with re == NULL to query npts only.
 */
int iris_get_fdata(iris_engine* eng, int box, int j, double* re, double* im, long* npts);

/* Run one operator group (IRIS_OP_*) for parity checks; arg is `it` for
 * IRIS_OP_TFSF and the DFT time index for IRIS_OP_DFT.  Returns
 * IRIS_ETIMEOUT when a bounded device wait gave up (the engine's error
 * word is cleared once reported, by any call that reports it). */
int iris_apply(iris_engine* eng, int op, int arg);

/*
 * Full drop-in run in directory dir: program IrisFDTD / main() / driver()
 * (code/program.f90:25-61, code/main.f90:43-213, code/driver.f90:66-555):
 * reads dir/inputFDTD.dat, writes log.dat and the <box>_scatt*.dat files
 * every no_downloads steps and at the last step.  precision: IRIS_FP64 or
 * IRIS_FP32.  The <<LOOP>> first line runs main() once per index.
 */
int iris_run_input(const char* dir, int precision);

/* ---- engine instrumentation (no reference counterpart) --------------- */
/* Kernel classes timed by iris_timing / iris_timing_read. */
#define IRIS_KC_E 0      /* E update (e_fdtd + UPML-E + Bloch max)        */
#define IRIS_KC_H 1      /* H update (h_fdtd + UPML-H + Bloch min)        */
#define IRIS_KC_TFSF 2   /* TF/SF source                                  */
#define IRIS_KC_GATHER 3 /* DFT face sample gather                        */
#define IRIS_KC_DFT 4    /* DFT block accumulation (and its twiddles)     */
#define IRIS_KC_FLUX 5   /* flux reduction                                */
#define IRIS_KC_FUSED 6  /* fused E+H pass (TF/SF and the DFT sample      */
                         /* follow as their own kernels)                  */
#define IRIS_KC_PERSIST 7 /* persistent kernel: a span of whole steps     */
#define IRIS_NKC 8

/*
 * Start a timed region on the engine's stream: records a start event and,
 * when enable != 0, a pair of CUDA events around every kernel launched
 * until iris_timing_read.
 */
int iris_timing(iris_engine* eng, int enable);
/* End the region: its device time, and per kernel class the summed device
 * time (ms) and the number of timed entries (arrays of IRIS_NKC, either may
 * be NULL): one per launch, except the plain engine's IRIS_KC_FUSED (one
 * per step) and the batch's flat work lists (one per E or H pass of two
 * launches). */
int iris_timing_read(iris_engine* eng, double* region_ms, double* kernel_ms, long* launches);
/* Sizes: info[0] DFT sample points, [1] DFT block length K, [2] bytes per
 * stored complex value, [3] elements per field component, [4] complex
 * material flag, [5] number of DFT boxes, [6] DFT samples buffered and not
 * yet accumulated into fdata (info: 7 entries). */
int iris_info(const iris_engine* eng, long* info);
/* Bounds-check record of the process's kernels.  Returns 1 when the library
 * was built with bounds checks (libiris_fdtd_bc.so, -DIRIS_BOUNDS_CHECK), 0
 * otherwise; *first receives the first out-of-range access any kernel met
 * since the last call, (site << 48) | index (0: none; sites: 1 E cell, 2 H
 * cell, 3 and 4 E and H UPML slab rows, 5 material, 6 TF/SF row, 7 and 8 DFT
 * sample source and slot, 9 and 10 fused-pass chunk and slab row, 11 and 12
 * DFT block point and sample, 13 flux face), and the record is cleared.  A
 * checked kernel skips the access it refuses.  No counterpart in the
 * reference (a Fortran build with -check bounds stops the program). */
int iris_bounds_check(unsigned long long* first);

/* ---- batched form ------------------------------------------------------ */
/*
 * Many independent Bloch cells (or k-points of one cell) stepped together;
 * no counterpart in the reference beyond its <<LOOP>> mode, which re-runs
 * main() per index (code/program.f90:36-57).  Each cell has its own grid,
 * UPML, structure, source plane, DFT box and Bloch phases; all cells share
 * the precision, Q, dt, the frequency list, the DFT sampling and the device.
 * One launch per operator covers every cell: persistent kernels walk a work
 * list of (cell, tile) items.  dft_faces: IRIS_DFT_ALL or IRIS_DFT_Z.
 */
typedef struct iris_batch iris_batch;
int iris_batch_create(int ncells, const iris_params* params, const double* fw, int dft_faces, iris_batch** out);
void iris_batch_destroy(iris_batch* b);
/* iris_set_material for one cell of the batch. */
int iris_batch_set_material(iris_batch* b, int cell, const double* eps_inv_re, const double* eps_inv_im);
/* iris_material_pattern for one cell of the batch. */
int iris_batch_material_pattern(iris_batch* b, int cell, unsigned long long seed, double fill, double eps_in,
                                double eps_out);
/* iris_step for every cell: steps it0 .. it0+nsteps-1. */
int iris_batch_step(iris_batch* b, int it0, int nsteps);
/* iris_flux (box 1) of one cell. */
int iris_batch_flux(iris_batch* b, int cell, double* J);
/* iris_dft_commit for every cell (they share one sample buffer). */
int iris_batch_dft_commit(iris_batch* b);
/* iris_get_field of one cell. */
int iris_batch_get_field(iris_batch* b, int cell, int which, double* re, double* im);
/*
 * Tile-shape autotuner: times every candidate work list (reps E+H passes,
 * or fused passes, each) on this batch and keeps the fastest; ms[i]
 * (optional, IRIS_BATCH_NTILES entries) receives the time per E+H pass of
 * candidate i (-1 for a candidate the precision does not offer).  Call
 * before the first step (the passes run on the zero initial state).
 */
#define IRIS_BATCH_NTILES 8
int iris_batch_tune(iris_batch* b, int reps, int* best, double* ms);
/* The autotuner with a cache by size class (the device, the precision, a
 * complex material, and the binary orders of magnitude of the cell count,
 * the total grid cells and the mean nx, ny, nz): a batch whose class was
 * tuned before in this process, or is listed in the file named by the
 * environment variable IRIS_TUNE_CACHE, takes the cached pick without
 * timing (*cached = 1); otherwise iris_batch_tune runs and its pick is
 * stored (and appended to that file).  Call before the first step. */
int iris_batch_autotune(iris_batch* b, int reps, int* best, int* cached);
/* Force a candidate work list (0..4: x*y*z blocks 32x8x1, 32x4x2, 64x4x1,
 * 16x16x1, 32x2x4 of the split E and H passes; 5, 6: runs of 256
 * consecutive cells of one plane, with registers capped for five resident
 * blocks per SM (5) or not (6); 7, FP32 only: the fused E+H pass over
 * 32x16 column tiles and z chunks, which first allocates every cell's
 * second field buffers (the fields then alternate between the two sets;
 * iris_batch_get_field always reads the current one)). */
int iris_batch_set_tile(iris_batch* b, int tile);
int iris_batch_timing(iris_batch* b, int enable);
int iris_batch_timing_read(iris_batch* b, double* region_ms, double* kernel_ms, long* launches);
/* info[0] cells, [1] total grid cells, [2] DFT points, [3] DFT block K,
 * [4] tile index, [5] work items per pass, [6] kernel launches per E or H
 * pass, or per fused pass, [7] DFT samples buffered and not yet accumulated
 * (info: 8 entries). */
int iris_batch_info(const iris_batch* b, long* info);

/* ---- adjoint (gradient) form ------------------------------------------- */
/*
 * dL/d(eps_inv) over a design region of the structure layer for the
 * objective
 *     L = sum_w  w5[w] * J5(w) + w6[w] * J6(w)
 * where J5 and J6 are the reflection and transmission fluxes of box 1
 * (the scattering_fourier_out numbers, code/dataprocess.f90:246-277).  No
 * counterpart in the reference: it differentiates the time loop that
 * code/driver.f90:338-451 runs.
 *
 * The gradient is the exact discrete adjoint of the engine's update: the
 * transposed E/H/UPML step run backwards in time with the conjugate-
 * transposed DFT as its source, accumulated against the forward curl of H
 * over the design cells.  Forward states are checkpointed every
 * checkpoint_every steps and each segment is recomputed from its checkpoint
 * during the backward sweep; the last segment's curls are recorded during the
 * forward solve itself, so checkpoint_every >= nsteps (one segment, curls of
 * every step kept: nsteps x 3 x design cells complex values) needs no
 * recompute.
 *
 * design: {x0, x1, y0, y1, z0, z1}, 1-based and inclusive, inside
 * [1,nx] x [1,ny] x [hi,hf].  weights: [2][nof] (w5 then w6), or NULL for
 * w5 = 0, w6 = 1.  The material must be real; the z planes of box 1 must lie
 * outside the UPML slabs (pmlzi < szi, szf < pmlzf).  Only box 1's z faces
 * are accumulated.
 */
typedef struct iris_adjoint iris_adjoint;
int iris_adjoint_create(const iris_params* p, const double* fw, const int design[6], int checkpoint_every,
                        const double* weights, iris_adjoint** out);
void iris_adjoint_destroy(iris_adjoint* a);
/* Whole structure material, as iris_set_material (imaginary part zero). */
int iris_adjoint_set_material(iris_adjoint* a, const double* eps_inv_re, const double* eps_inv_im);
/* eps_inv of the design cells, [z][y][x] with x fastest. */
int iris_adjoint_set_design(iris_adjoint* a, const double* eps_inv);
/* Forward solve from zero fields over steps 1..nsteps, saving checkpoints;
 * L receives the objective, J (optional, [6][nof]) the box-1 fluxes. */
int iris_adjoint_forward(iris_adjoint* a, int nsteps, double* L, double* J);
/* Backward sweep for the last forward: grad[z][y][x] = dL/d eps_inv. */
int iris_adjoint_backward(iris_adjoint* a, double* grad);
/* The forward engine (which = 0) or the engine holding the adjoint state
 * (which = 1: E, H, D, B read and written with iris_get/set_field and
 * iris_get/set_pml).  Borrowed: owned by the adjoint object. */
int iris_adjoint_engine(iris_adjoint* a, int which, iris_engine** eng);
/* nsteps steps of the homogeneous adjoint recursion (no sources, no
 * gradient) applied to the adjoint state, for a step at time index it: the
 * conjugate transpose of nsteps source-free forward steps. */
int iris_adjoint_apply(iris_adjoint* a, int nsteps);
/* Device time (ms) of the last forward, of the last backward's recompute
 * and of its adjoint sweep; ms[3]. */
int iris_adjoint_timing(const iris_adjoint* a, double* ms);

/* ---- allocation-free DFT block ---------------------------------------- */
/*
 * This entry point has no counterpart in the reference.  It exists for
 * callers that cannot call cudaMalloc while they run: a host code whose
 * device memory is owned by a pooling allocator (a framework's caching
 * allocator, a buffer pool registered once for communication) or a
 * deployment that forbids device allocation after start-up.  Such a caller
 * cannot create an engine (iris_create allocates), but can still run the
 * engine's FP32 DFT block accumulation on buffers it already owns.
 *
 * It adds nk samples to caller-owned accumulators, on the caller's stream:
 *   fdata[iw][p] += sum_k samples[k][p] * dt * exp(i*fw[iw]*(t0 + k*t_step))
 * with the partial sum over the block in FP32 and one FP64 add per
 * (p, iw), exactly like the engine's FP32 mode.  All pointers are device
 * pointers owned by the caller: samples [nk][npts] complex float (re, im
 * interleaved), fw [nof] double, fdata [nof][npts] complex double.
 * stream is a cudaStream_t (NULL: the legacy default stream).
 *
 * It allocates nothing.  The twiddle table it needs lives in a fixed device
 * array of IRIS_NOALLOC_MAX_TWIDDLES complex floats (512 KiB) that every
 * GPU which loads the library holds until the process exits; calls with
 * nk*nof above that are rejected with IRIS_EINVAL (split the block).  The
 * first call on each device looks up that array's device address (a
 * one-time set-up per device, made with the caller's current device); make
 * that first call before any stream capture.  The address is kept for the
 * life of the process: it does not survive cudaDeviceReset or the teardown
 * of the device's primary context, after which this entry point must not be
 * called again in that process.  Every call reuses the same array and
 * overwrites the entries it uses, so nothing needs clearing, but calls whose
 * kernels overlap on the GPU (different streams, no ordering) race on it.
 * samples and fw must be 8-byte aligned and fdata 16-byte aligned.  Every
 * argument is checked before any CUDA call, so a refused call touches no
 * device.  A CUDA error still pending from earlier work on the calling
 * thread is returned as IRIS_ECUDA (with its text) and nothing is launched.
 * Returns before the kernels finish; errors of the launches are reported,
 * errors of their execution surface at the next sync.
 */
#define IRIS_NOALLOC_MAX_TWIDDLES 65536
int iris_dft_block_noalloc(const void* samples, int nk, long npts, int t0, int t_step,
                           const double* fw, int nof, double dt, void* fdata, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* IRIS_FDTD_H */
