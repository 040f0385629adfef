/*
 * mhdgpu.h - C ABI of the GB300 (sm_103a) implementation of one dimensionally
 * split step of Pen's relaxing TVD MHD solver.
 *
 * Data layout (identical to the reference, Heterogeneous_MHD/C/array_definition.h:12-14):
 *   u(5,nx,ny,nz) = (rho, m_x, m_y, m_z, E) and b(3,nx,ny,nz), FP32, component
 *   fastest, then i, j, k.  b is face-centred on the left faces of each cell.
 * Every subroutine works in the frame it is called with: the pencil runs along
 * the first spatial axis (length nx), its neighbours are j+-1 and k+-1.
 *
 * Conventions of this ABI:
 *   - plain pointers and sizes; device pointers unless a name says host;
 *   - every entry returns an int status (MHD_OK on success) and never exits
 *     or traps; mhdgpu_last_error() gives a message for the calling thread;
 *   - the device entries are asynchronous on the given stream (NULL = legacy
 *     default stream), allocate nothing and can be captured in a CUDA graph;
 *   - the caller owns every buffer, scratch included (sizes from the
 *     *_bytes queries); the library keeps no per-call state, so calls are
 *     re-entrant on different streams.
 *
 * Citations are files of pandaPQY/MHD-GPU.
 */
#ifndef MHDGPU_H
#define MHDGPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* cudaStream_t without including the CUDA headers */
typedef struct CUstream_st *mhdgpu_stream_t;

/* status codes */
#define MHD_OK              0
#define MHD_ERR_ARG         1   /* bad size, null pointer, aliasing, unsupported shape */
#define MHD_ERR_CUDA        2   /* a CUDA runtime call failed */
#define MHD_ERR_TIMEOUT     3   /* a bounded device wait gave up */
#define MHD_ERR_UNPHYSICAL  4   /* the health word reports NaN/Inf or rho<=0 */
#define MHD_ERR_NOMEM       5   /* a host-buffer entry could not allocate */

/* CFL formulas */
#define MHD_CFL_C           0   /* C path: the cell's own face B, unaveraged
                                   (Heterogeneous_MHD/C/calcfl.c:13-65) */
#define MHD_CFL_AVERAGED    1   /* release 0.2: B averaged to the cell centre
                                   (OpenMP/mhd.f90:96-125, Cuda/cuda_cfl.cu:101-124) */

/* device health word bits (OR-ed by the kernels, read by the host) */
#define MHD_HEALTH_NONFINITE 1u  /* NaN or Inf in an updated state */
#define MHD_HEALTH_DENSITY   2u  /* rho <= 0 */
#define MHD_HEALTH_PRESSURE  4u  /* gas pressure <= 0 at the RK2 full step: a warning.
                                    In FP32 the recovery p = ps - B^2/2 cancels at low
                                    plasma beta and dips below 0 at round-off; the
                                    reference solver runs through it (it takes |.| in
                                    the fast speed, C/mhdflux.c:45), and so does this
                                    one.  Only NONFINITE and DENSITY fail a run. */
#define MHD_HEALTH_STALL     8u  /* batched kernel: a dependency wait gave up (about
                                    two seconds); the batch's state is invalid */

/* largest pencil the device kernels accept (cells along the frame's x) */
#define MHD_MAX_PENCIL      1024

const char *mhdgpu_status_string(int status);
const char *mhdgpu_last_error(void);
const char *mhdgpu_version(void);

/* ------------------------------------------------------------------------
 * Per-subroutine device API.  These replace the reference CUDA wrappers of
 * Heterogeneous_MHD/Cuda/cuda_subroutine.h:4-12 (which took the sizes both as
 * host and device int* and synchronised after every call).
 * ------------------------------------------------------------------------ */

/* fluidx: relaxing-TVD RK2 update of u along the pencil with cell-centred B.
 * Reads u_in and b (b at j+1 and k+1 for the transverse averages), writes
 * u_out; u_out == u_in is allowed (in place).  dt is read from device memory.
 * Replaces Cuda/cuda_fluidx.cu:12-23 and C/fluidx.c:19-102 (+ tvd1.c,
 * mhdflux.c).  health may be NULL. */
int mhdgpu_fluidx(float *u_out, const float *u_in, const float *b,
                  int nx, int ny, int nz, const float *d_dt,
                  unsigned *d_health, mhdgpu_stream_t stream);

/* advectbyzx: constrained-transport advection of the two transverse face
 * fields along the pencil, in place on b.  Needs caller scratch of
 * mhdgpu_advectbyzx_scratch_bytes() (two floats per cell).
 * Replaces Cuda/cuda_advectbyzx.cu:15-29 and C/advectbyzx.c:14-23
 * (+ advectbyzxA1/A2/B1/B2.c, tvdb.c). */
size_t mhdgpu_advectbyzx_scratch_bytes(int nx, int ny, int nz);
int mhdgpu_advectbyzx(float *b, const float *u, int nx, int ny, int nz,
                      const float *d_dt, float *d_scratch, mhdgpu_stream_t stream);

/* advectbyzx for callers that cannot allocate device memory.  No counterpart
 * in the reference (whose CUDA wrapper takes caller scratch, d_temp).
 * Same result as mhdgpu_advectbyzx, but the two floats of scratch per cell
 * come from a fixed array inside the library (MHD_NOALLOC_MAX_CELLS * 8
 * bytes = 16 MiB, held on every GPU that loads the library until exit), so a
 * caller that owns only its inputs and outputs -- a plugin running inside
 * another runtime's memory pool, or a loop that must not allocate -- can run
 * it.  It allocates nothing.  Boxes above MHD_NOALLOC_MAX_CELLS cells are
 * rejected with MHD_ERR_ARG.  The first call on a device looks up the array's
 * device address with that device current; make it before any stream
 * capture.  mhdgpu_release_host_cache forgets those addresses: call it before
 * a device reset, and the next call on the device looks the address up again
 * (so that call, too, must come before any capture).  All calls share the array, so calls that overlap on the GPU race
 * and must be serialised by the caller.  Nothing in the array has to start at
 * zero: each call writes every entry it reads. */
#define MHD_NOALLOC_MAX_CELLS 2097152   /* 128^3 */
int mhdgpu_advectbyzx_noalloc(float *b, const float *u, int nx, int ny, int nz,
                              const float *d_dt, mhdgpu_stream_t stream);

/* transpose12: (nx,ny,nz) -> (ny,nx,nz), u components (1,3,2,4,5) and b
 * components (2,1,3) (1-based).  Out of place; bit-exact.
 * Replaces Cuda/cuda_transpose12.cu:12-38 and C/transpose12.c:7-47. */
int mhdgpu_transpose12(float *dst_u, float *dst_b, const float *src_u, const float *src_b,
                       int nx, int ny, int nz, mhdgpu_stream_t stream);

/* transpose13: (nx,ny,nz) -> (nz,ny,nx), u components (1,4,3,2,5) and b
 * components (3,2,1).  Out of place; bit-exact.  Unlike the reference
 * (C/transpose13.c:16,58-61 refuses nx != nz) every shape is accepted.
 * Replaces Cuda/cuda_transpose13.cu:14-55 and C/transpose13.c:9-62. */
int mhdgpu_transpose13(float *dst_u, float *dst_b, const float *src_u, const float *src_b,
                       int nx, int ny, int nz, mhdgpu_stream_t stream);

/* cfl: writes 1/c_max to *d_inv_c, c_max = max over cells of the fast speed
 * (mode MHD_CFL_C or MHD_CFL_AVERAGED).  d_scratch is one unsigned word.
 * Replaces Cuda/cuda_cfl.cu:14-50 (whose result made a host round trip) and
 * C/calcfl.c:13-65 (whose return value is 1/c). */
int mhdgpu_cfl(const float *u, const float *b, int nx, int ny, int nz, int mode,
               float *d_inv_c, unsigned *d_scratch, mhdgpu_stream_t stream);

/* dt update of the driver (C/mhd.c:63-65) on the device:
 *   dt = (float)(cfl_number * (double)inv_c); if tf > 0 and dt > (tf - t)/2
 *   then dt = (tf - t)/2; t = t + 2*dt.  tf <= 0 disables the clamp. */
int mhdgpu_dt_update(const float *d_inv_c, double cfl_number, float tf,
                     float *d_t, float *d_dt, mhdgpu_stream_t stream);

/* copy_matrix (C/copy_matrix.c:9-38): update <- (u, b). */
int mhdgpu_copy_matrix(float *dst_u, float *dst_b, const float *src_u, const float *src_b,
                       int nx, int ny, int nz, mhdgpu_stream_t stream);

/* ------------------------------------------------------------------------
 * Whole step.  The sequence is the reference's Strang-symmetric
 * x, y(T12), z(T13), z, y(T13), x(T12) (C/mhd.c:72-119) built from the
 * per-subroutine kernels above, with the transposes ping-ponging between the
 * state and the workspace instead of the reference's copy_matrix calls.
 * ------------------------------------------------------------------------ */

/* workspace for mhdgpu_step / mhdgpu_advance (40 bytes per cell) */
size_t mhdgpu_step_workspace_bytes(int nx, int ny, int nz);

/* one full step at the dt held in *d_dt, in place on (u, b) */
int mhdgpu_step(float *u, float *b, int nx, int ny, int nz, const float *d_dt,
                void *d_work, unsigned *d_health, mhdgpu_stream_t stream);

/* The same step without transposes: the y and z sweeps read and write their
 * pencils in place in the x-major state through strided views (the frames of
 * C/mhd.c:79-113 after transpose12/13), so no data moves between sweeps.  Each
 * sweep is a fluid kernel, a field-advection kernel and a b(1) gather; the
 * arithmetic per pencil is that of mhdgpu_step, bit for bit.  Workspace:
 * mhdgpu_step_fused_workspace_bytes (8 bytes per cell). */
size_t mhdgpu_step_fused_workspace_bytes(int nx, int ny, int nz);
int mhdgpu_step_fused(float *u, float *b, int nx, int ny, int nz, const float *d_dt,
                      void *d_work, unsigned *d_health, mhdgpu_stream_t stream);

#define MHD_PATH_PLAIN      0   /* mhdgpu_step: per-subroutine kernels + transposes */
#define MHD_PATH_FUSED      1   /* mhdgpu_step_fused: transpose-free */
#define MHD_PATH_AUTO       2   /* the faster of the two for the box (mhdgpu_resolve_path) */

/* The path MHD_PATH_AUTO takes for an nx*ny*nz box: MHD_PATH_FUSED when
 * every y and z pencil has at most 48 cells, else MHD_PATH_PLAIN (measured
 * on GB300 with default tiles: the transpose-free step takes 0.82-0.89 of
 * the plain step's time at 32^3, 48^3 and 128x32x32, the same at 64^3 and
 * 96^3, and 1.03-1.10 of it from 128^3 up and wherever a y or z pencil is 64
 * cells or longer in a larger box; the plain step's transposes run near the
 * copy bandwidth and leave every sweep on contiguous pencils).
 * mhdgpu_path_workspace_bytes sizes the workspace of a path (MHD_PATH_AUTO:
 * of the path it takes). */
int mhdgpu_resolve_path(int nx, int ny, int nz);
size_t mhdgpu_path_workspace_bytes(int nx, int ny, int nz, int path);

/* clock of a run kept on the device */
typedef struct {
    float t;        /* simulation time */
    float dt;       /* dt of the last step */
    float inv_c;    /* 1/c_max of the last CFL evaluation */
    unsigned cmax;  /* CFL reduction word: between steps, the fast speed of the
                       current state folded in by the last sweep (float bits) */
    unsigned health;/* MHD_HEALTH_* bits */
    int iter;       /* steps taken */
} mhdgpu_clock;

/* nsteps iterations of: CFL -> dt update -> step, all on the device
 * (C/mhd.c:60-125 without its printfs).  d_dt_log (may be NULL) receives each
 * step's dt at d_dt_log[clock.iter], so it must hold clock.iter + nsteps
 * entries.  Steps with tf > 0 and t >= tf are skipped on the device (the
 * reference's do-while exit).  path = MHD_PATH_PLAIN (d_work of
 * mhdgpu_step_workspace_bytes), MHD_PATH_AUTO (of mhdgpu_path_workspace_bytes)
 * or MHD_PATH_FUSED (of
 * mhdgpu_step_fused_workspace_bytes).
 *
 * The CFL reduction runs as its own pass over the state before the call's
 * first step (on a cleared word, so a state written since the clock's last
 * step takes its own speed); each step's last fluid sweep folds the next step's reduction
 * into the clock's CFL word, so later steps of the call need no pass.  With
 * MHD_ADVANCE_RESUME or'ed into cfl_mode, the first step takes that folded
 * word too: valid only when the clock's last step was taken by mhdgpu_advance
 * on this same state and the state is unchanged since (a run driven one step
 * per call, e.g. one step per CUDA graph launch). */
#define MHD_ADVANCE_RESUME 0x100
int mhdgpu_advance(float *u, float *b, int nx, int ny, int nz, int nsteps,
                   double cfl_number, int cfl_mode, float tf,
                   mhdgpu_clock *d_clock, float *d_dt_log, void *d_work,
                   int path, mhdgpu_stream_t stream);

/* ------------------------------------------------------------------------
 * Host-buffer entry (the end-to-end path): uploads (u, b) from host memory,
 * runs up to max_steps steps as mhdgpu_advance does, downloads the state.
 * Its device buffers and stream are kept per host thread between calls
 * (grown to the largest box seen; mhdgpu_release_host_cache frees them, and
 * they are freed when the thread ends).  *t is read and updated; dt_log may
 * be NULL.  Returns the steps taken in *steps_done (may be NULL).  path as
 * for mhdgpu_advance.
 * ------------------------------------------------------------------------ */
int mhdgpu_run_host(float *u, float *b, int nx, int ny, int nz, double cfl_number,
                    int cfl_mode, float *t, float tf, int max_steps, float *dt_log,
                    int *steps_done, int path);
/* Frees the calling thread's device buffers and stream of mhdgpu_run_host,
 * and drops the device addresses that mhdgpu_advectbyzx_noalloc looked up
 * (call it before resetting the device from that thread). */
int mhdgpu_release_host_cache(void);

/* ------------------------------------------------------------------------
 * Arithmetic policy and row staging (settings of the calling host thread:
 * a setting made on one thread changes only the launches that thread makes,
 * and a CUDA graph keeps the settings it was captured with), and tile shapes
 * (a process-wide table; a shape changes the speed, never the result).
 * ------------------------------------------------------------------------ */
#define MHD_MATH_FAITHFUL   0   /* rounding of the reference C path (default) */
#define MHD_MATH_FAST       1   /* plain FP32 with FMA contraction, hardware
                                   reciprocal and root: faster, ~1 ulp per op
                                   further from the reference */
#define MHD_MATH_FP64P      2   /* faithful, except that the gas pressure of
                                   low-beta cells (beta = 2p/B^2 < 0.1 in FP32,
                                   or p <= 0) is recovered in FP64:
                                   p = (gamma-1)(E - m^2/2rho - B^2/2) from the
                                   float state in double (the reference forms
                                   ps first and p = ps - B^2/2, which cancels
                                   at low beta, C/mhdflux.c:26-42) */

/* selects the policy of the fluid kernels; returns the previous one */
int mhdgpu_set_math(int mode);

/* How the transpose-free step moves the pencils that run across memory (its
 * y and z sweeps) between global and shared memory:
 *   MHD_STAGING_CPASYNC (default): a full tile of the fluid sweep (every row
 *     stride a multiple of 4 cells, 16-byte aligned arrays, pencils per CTA a
 *     multiple of 4) is moved as 16-byte vectors of four pencils' cells per
 *     thread; partial tiles and the field sweep's tiles row by row with
 *     4-byte asynchronous copies;
 *   MHD_STAGING_TMA: where the frame allows (pencils of 32, 64 or 128 cells in
 *     teams of one warp, 8 per CTA, every row stride a multiple of 4 cells,
 *     16-byte aligned arrays) the fluid tile is loaded and stored by tensor
 *     copies of the Tensor Memory Accelerator, with the component transpose
 *     done in shared memory.
 * Both give the same bits (the batch always takes the first).  Returns the
 * previous mode (-1 for a bad mode). */
#define MHD_STAGING_TMA      0
#define MHD_STAGING_CPASYNC  1
int mhdgpu_set_row_staging(int mode);

/* Poison mode, a debugging aid: with on != 0 every entry that takes scratch
 * (mhdgpu_advectbyzx, mhdgpu_step, mhdgpu_step_fused and so mhdgpu_advance,
 * the batch's steps) first fills it with NaN on its stream, so a kernel that
 * read scratch before writing it would put NaN into the state.  Results are
 * unchanged otherwise; it costs one memset per call.  Returns the previous
 * setting (of the calling host thread). */
int mhdgpu_set_poison(int on);

/* Debug build (lib/libmhdgpu_debug.so, build.py --debug): every shared-memory,
 * global and halo index of the kernels is checked where it is formed; an
 * index outside its array is skipped (a load reads 0, a store or copy does not
 * happen) and recorded.  mhdgpu_debug_build returns 1 in that build, 0 in the
 * release build.  mhdgpu_debug_faults synchronises the device, reports the
 * number of faults since the last call and the first one (kind 1: an index
 * into an array, 2: shared memory outside the launch's dynamic area, 3: a
 * global array; the source file's number in the debug build's table and the
 * line; the index or offset and the extent it broke) and clears the count.
 * In the release build it reports 0 faults.  Any pointer may be NULL.
 * File numbers: 1 fluidx_reg.cuh, 2 fluidx_kernel.cuh, 3 advect_reg.cuh,
 * 4 advect_kernel.cuh, 5 batch_kernel.cuh, 6 transpose.cu, 7 cfl_kernel.cuh,
 * 8 tma_rows.cuh, 9 mhd_common.cuh, 10 debug.cu.
 * mhdgpu_debug_selftest checks index against extent in a one-thread kernel
 * (nothing is accessed through the index) and returns in *in_bounds whether
 * the check passed: the debug build records a failed check like any other;
 * the release build has no checks and always reports 1. */
int mhdgpu_debug_build(void);
int mhdgpu_debug_faults(unsigned *count, unsigned *kind, unsigned *file, unsigned *line,
                        long long *index, long long *extent);
int mhdgpu_debug_selftest(long long index, long long extent, int *in_bounds);

/* Team shape of a pencil kernel (kclass MHD_KCLASS_FLUIDX or
 * MHD_KCLASS_ADVECT, OR-ed with MHD_TILE_ROWS for pencils that run across
 * memory -- the y and z sweeps of mhdgpu_step_fused) for pencils of length n:
 * cpl cells per thread, wpp warps per pencil, ppc pencils per CTA;
 * n <= 32*wpp*cpl and 32*wpp*ppc <= 256.  mhdgpu_set_tile overrides the
 * default table; mhdgpu_get_tile reports the shape in use.  The table is per
 * host thread, like the settings above (mhdgpu_autotune and
 * mhdgpu_tile_cache_load fill the calling thread's).  Compiled shapes
 * (cpl,wpp): (1,1) (2,1) (4,1) (1,2) (2,2) (4,2) (1,4) (2,4) (4,4) (2,8) (4,8). */
#define MHD_TILE_ROWS       16
int mhdgpu_set_tile(int kclass, int n, int cpl, int wpp, int ppc);
int mhdgpu_get_tile(int kclass, int n, int *cpl, int *wpp, int *ppc);

/* Autotuner: for each pencil length the step uses on an nx*ny*nz box (nx, ny
 * and nz), times every compiled shape of the fluid and advection kernels on a
 * synthetic state of this box with CUDA events, keeps the fastest through
 * mhdgpu_set_tile and returns.  Allocates and frees its own test buffers;
 * synchronises the device.  Not for use under stream capture. */
int mhdgpu_autotune(int nx, int ny, int nz, int math);

/* The autotuner's picks as JSON, so a tuned configuration is reused without
 * timing it again.  mhdgpu_tile_cache_save writes every shape set in this
 * process's table (by mhdgpu_set_tile or mhdgpu_autotune) with the current
 * device's name; mhdgpu_tile_cache_load sets the shapes a file holds and
 * reports how many in *applied (0 when the file was written on another
 * device model).  MHD_ERR_ARG for an unreadable or malformed file. */
int mhdgpu_tile_cache_save(const char *path);
int mhdgpu_tile_cache_load(const char *path, int *applied);

/* ------------------------------------------------------------------------
 * FP64 diagnostics of a state (the reference prints float sums from the host,
 * Heterogeneous_MHD/C/check_value.c:22-79).  d_out (device, 8 doubles):
 *   [0..4] sums of rho, m_x, m_y, m_z, E over the box;
 *   [5]    max |div B| = |b1(i+1)-b1(i) + b2(j+1)-b2(j) + b3(k+1)-b3(k)|;
 *   [6]    min gas pressure p = (gamma-1)(E - m^2/2rho - Bc^2/2), Bc the
 *          face field averaged to the cell centre as fluidx does;
 *   [7]    number of cells with p <= 0.
 * Every term and partial sum is a double; the order is fixed by the box size,
 * so results repeat bit for bit.  d_scratch holds
 * mhdgpu_diagnostics_scratch_bytes(nx, ny, nz) bytes (<= 40 KB).
 * ------------------------------------------------------------------------ */
#define MHD_DIAG_COUNT 8
size_t mhdgpu_diagnostics_scratch_bytes(int nx, int ny, int nz);
int mhdgpu_diagnostics(const float *u, const float *b, int nx, int ny, int nz, double *d_out,
                       void *d_scratch, mhdgpu_stream_t stream);

/* ------------------------------------------------------------------------
 * State files in the reference's formats (host arrays in the reference
 * layout; the reference hard-codes sizes and file names, these take both):
 *   mhdgpu_read_state / mhdgpu_write_state: the init file of
 *     Heterogeneous_MHD/C/init.c:33-66 -- raw float32, cells x-outer,
 *     z-inner, 8 floats each (rho, m_x, m_y, m_z, E, b_x, b_y, b_z); a run
 *     checkpoints with write_state and resumes with read_state;
 *   mhdgpu_write_result: the final dump of C/mhd.c:126-160 -- two raw files,
 *     u (5 floats per cell) and b (3), cells x-outer, z-inner;
 *   mhdgpu_write_check: the check dump of C/check_value.c:22-79 -- eight text
 *     files <prefix>u1.dat .. <prefix>b3.dat, "%8.6e" per line, x fastest.
 * MHD_ERR_ARG on bad arguments or a file of the wrong size, MHD_ERR_NOMEM on
 * an I/O failure.
 * ------------------------------------------------------------------------ */
int mhdgpu_read_state(const char *path, float *u, float *b, int nx, int ny, int nz);
int mhdgpu_write_state(const char *path, const float *u, const float *b, int nx, int ny, int nz);
int mhdgpu_write_result(const char *path_u, const char *path_b, const float *u, const float *b,
                        int nx, int ny, int nz);
int mhdgpu_write_check(const char *prefix, const float *u, const float *b, int nx, int ny, int nz);

/* ------------------------------------------------------------------------
 * Batched ensemble (no counterpart in the reference, whose drivers advance
 * one box: Heterogeneous_MHD/C/mhd.c:59-125).  Many independent periodic
 * boxes, each with its own sizes (1 .. MHD_BATCH_MAX_PENCIL cells on every
 * axis; non-cubic and uneven allowed), state, clock and dt, advance together.
 * A step is one clock launch and, per sweep (x, y, z, z, y, x), one
 * persistent launch per pencil-length class present (the boxes whose pencils
 * along the sweep share a team shape; at most 64 boxes per launch), the
 * classes of a sweep running concurrently on side streams; the CFL reduction
 * runs once per mhdgpu_batch_advance call and is otherwise folded into each
 * step's last sweep.  Each box goes through the transpose-free step of
 * mhdgpu_step_fused and ends bit for bit where
 * mhdgpu_advance(path = MHD_PATH_FUSED) takes it alone.
 *
 * The state of box i stays in the caller's device arrays d_u[i] (5 floats
 * per cell) and d_b[i] (3 per cell), reference layout; the handle keeps the
 * pointers.  mhdgpu_batch_create allocates the handle's device memory
 * (mhdgpu_batch_workspace_bytes: 8 bytes per cell plus small tables) and
 * synchronises; nothing else allocates.  tf (host, nbox floats, or NULL for
 * none) is each box's end time, with the dt clamp and dt = 0 after the end as
 * in mhdgpu_advance.  Clocks start at t = 0.
 * ------------------------------------------------------------------------ */
#define MHD_BATCH_MAX_PENCIL 256
#define MHD_BATCH_MAX_BOXES  65536

typedef struct mhdgpu_batch mhdgpu_batch;
size_t mhdgpu_batch_workspace_bytes(int nbox, const int *dims /* 3*nbox: nx,ny,nz */);
int mhdgpu_batch_create(mhdgpu_batch **out, int nbox, const int *dims, float *const *d_u,
                        float *const *d_b, double cfl_number, int cfl_mode, const float *tf);
int mhdgpu_batch_destroy(mhdgpu_batch *bt);
/* enqueues nsteps steps on stream (capturable into a CUDA graph, no host
 * synchronisation; the side streams fork from and join back to stream) */
int mhdgpu_batch_advance(mhdgpu_batch *bt, int nsteps, mhdgpu_stream_t stream);
/* as mhdgpu_batch_advance, continuing the handle's previous advance: the first
 * step takes the CFL speeds folded into the previous step's last sweep instead
 * of a reduction pass.  Valid only when no box's state changed since the
 * handle's last advance; the handle runs the pass anyway when it has not
 * advanced yet (mhdgpu_batch_tune puts the clock records, folded speeds
 * included, back as they were). */
int mhdgpu_batch_resume(mhdgpu_batch *bt, int nsteps, mhdgpu_stream_t stream);
/* The host-buffer entry of the ensemble: uploads every box from h_u[i]
 * (5 floats per cell) and h_b[i] (3 per cell), advances nsteps steps as
 * mhdgpu_batch_advance does, downloads the boxes into the same buffers and
 * synchronises stream.  With two boxes or more the boxes are split into up to
 * four parts of about equal cells, pipelined on the handle's side streams:
 * a part steps as soon as its boxes are uploaded while the next part uploads,
 * and downloads while later parts still step (the parts are built on the
 * first call, with the handle's schedule).  Results equal the device path's
 * bit for bit.  Pinned host buffers copy fastest.  The boxes' device arrays
 * given at creation are overwritten. */
int mhdgpu_batch_run_host(mhdgpu_batch *bt, float *const *h_u, float *const *h_b, int nsteps,
                          mhdgpu_stream_t stream);
/* synchronises stream and copies the nbox clocks to the host; returns
 * MHD_ERR_TIMEOUT after a stall, MHD_ERR_UNPHYSICAL when a box's health
 * reports NaN/Inf or rho <= 0 */
int mhdgpu_batch_read_clocks(mhdgpu_batch *bt, mhdgpu_clock *clocks, mhdgpu_stream_t stream);
/* Block schedule of the sweeps along one axis (0, 1, 2): threads per CTA
 * (64, 128 or 256; a CTA holds threads/32 pencils of length <= 128 or half as
 * many longer ones) and resident CTAs per SM (the persistent grid is
 * SMs x ctas_per_sm, capped by the occupancy the kernel allows).  Synchronous:
 * waits for the device's queued work, then uploads the work tables; not under
 * stream capture.  A CUDA graph captured from this handle's steps before a
 * schedule change (this call or mhdgpu_batch_tune) keeps the old launch shapes
 * and must be captured again. */
int mhdgpu_batch_set_schedule(mhdgpu_batch *bt, int axis, int threads, int ctas_per_sm);
int mhdgpu_batch_get_schedule(const mhdgpu_batch *bt, int axis, int *threads, int *ctas_per_sm);
/* Autotuner: times every schedule on this batch's own boxes (one warm-up and
 * four timed steps each, CUDA events per sweep), keeps the fastest per axis and
 * restores the boxes' state and clocks.  Allocates a snapshot of the state
 * for the duration; waits for the device's queued work (steps of this handle
 * already enqueued on any stream finish first); synchronises.  Not under
 * stream capture. */
int mhdgpu_batch_tune(mhdgpu_batch *bt, mhdgpu_stream_t stream);

/* The batch's schedule (threads and CTAs-per-SM cap of each axis, e.g. as
 * mhdgpu_batch_tune left it) as JSON, with the device's name and a signature
 * of the batch (its boxes' sizes in order and the calling thread's arithmetic
 * policy).  mhdgpu_batch_schedule_load applies a file's schedule when device
 * and signature match (*applied = 1; a schedule change as by
 * mhdgpu_batch_set_schedule), else leaves the batch as it is (*applied = 0). */
int mhdgpu_batch_schedule_save(const mhdgpu_batch *bt, const char *path);
int mhdgpu_batch_schedule_load(mhdgpu_batch *bt, const char *path, int *applied);
/* Failure-path test hook: from the next step on, the first dependency wait of
 * box 0 in the first sweep waits for one item more than exist, so it gives up
 * after its limit (about two seconds): the box's health gets MHD_HEALTH_STALL,
 * the batch's later waits return at once, the launches drain and
 * mhdgpu_batch_read_clocks returns MHD_ERR_TIMEOUT.  The batch's state is then
 * invalid; the context stays usable. */
int mhdgpu_batch_inject_stall(mhdgpu_batch *bt);

/* ------------------------------------------------------------------------
 * Profiler: per-kernel-class device time from CUDA events.  While a profiler
 * is attached to the calling thread, every entry above records a start and
 * an end event on its stream around its launches (no added synchronisation;
 * not for use under stream capture).  The reference timed whole steps only
 * (Cuda/cuda_main.cu:68-77,122-128).
 * ------------------------------------------------------------------------ */
#define MHD_KCLASS_FLUIDX     0   /* fluidx kernel */
#define MHD_KCLASS_ADVECT     1   /* advectbyzx flux kernel + b_x gather kernel */
#define MHD_KCLASS_TRANSPOSE  2   /* transpose12 / transpose13 */
#define MHD_KCLASS_CFL        3   /* CFL reduction (+ its clock/finish kernel) */
#define MHD_KCLASS_BATCH      4   /* batched ensemble sweeps (mhdgpu_batch_advance) */
#define MHD_KCLASS_COUNT      5

typedef struct mhdgpu_profiler mhdgpu_profiler;
int mhdgpu_profiler_create(mhdgpu_profiler **p, int max_records);
int mhdgpu_profiler_destroy(mhdgpu_profiler *p);
/* attach to the calling thread; NULL detaches */
int mhdgpu_profiler_attach(mhdgpu_profiler *p);
int mhdgpu_profiler_reset(mhdgpu_profiler *p);
/* waits for the recorded events of one class; records = timed regions,
 * launches = kernels launched inside them, total_ms = summed device time */
int mhdgpu_profiler_summary(mhdgpu_profiler *p, int kclass, int *records, int *launches,
                            double *total_ms);

#ifdef __cplusplus
}
#endif

#endif /* MHDGPU_H */
