/*
 * cliffs_gpu.h -- C ABI of the GB300 (sm_103a) Cliffs time-stepping library.
 *
 * Drop-in for the hot path of the Cliffs tsunami model: the loop body of
 * cliffs_main.f:303-378 (x- and y-sweeps of subroutine cliffs, cliffs.f:17-346;
 * the max-wave update; the nested-grid feed; gauge and screenshot sampling).
 * The Fortran driver keeps its setup and NetCDF I/O and calls these entry
 * points through ISO_C_BINDING; fields stay resident on one GPU between
 * output intervals.
 *
 * Conventions
 *  - Every 2-D array is column-major (x fastest) exactly like the Fortran
 *    module arrays: element (i,j), 1-based, at [(i-1) + (j-1)*nx].
 *  - Grid indices passed in (gauges, nest tables, records) are 1-based.
 *  - Every call returns an int status: CLIFFS_OK (0) on success, a positive
 *    informational code, or a negative error code; nothing in the library
 *    calls exit().  cliffs_gpu_strerror() names a code.
 *  - One context is driven by one host thread at a time; calls on a context
 *    are ordered on its CUDA stream.  Independent contexts (ensembles,
 *    parent/child grids) may share a device.
 */
#ifndef CLIFFS_GPU_H
#define CLIFFS_GPU_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  CLIFFS_OK = 0,
  CLIFFS_FEED_ENDED = 1,      /* forcing ended with freeze set (cliffs_main.f:305-311) */
  CLIFFS_WARN_CFL = 2,        /* a sweep read a state whose Courant number exceeds 1 */
  CLIFFS_ERR_ARG = -1,        /* bad argument or grid description */
  CLIFFS_ERR_CUDA = -2,       /* CUDA runtime error */
  CLIFFS_ERR_NAN = -3,        /* a non-finite eta/u/v appeared */
  CLIFFS_ERR_NOMEM = -4,      /* device allocation failed */
  CLIFFS_ERR_STATE = -5,      /* call out of order (e.g. no state uploaded) */
  CLIFFS_ERR_DEVICE = -6,     /* no usable sm_103 device */
  CLIFFS_ERR_TIMEOUT = -7     /* a device-side wait ran out (batch barrier, sweep stage) */
};

/* status bits reported by cliffs_gpu_status() */
enum {
  CLIFFS_ST_NAN = 1u,         /* a sweep produced a non-finite value */
  CLIFFS_ST_STALL = 2u,       /* a staged sweep's shared-memory stage wait ran out */
  CLIFFS_ST_CFL = 4u          /* a sweep read a cell whose Courant number
                                 (|u|+c) dt / ((dx(m-1)+dx(m))/2) exceeds 1 */
};

typedef struct cliffs_ctx cliffs_ctx;

/* Grid and physical parameters of one Cliffs grid (modules MASTER and
 * PARAMETERS, global_modules.f:16-55, as filled by allabout.f and
 * MasterGrid.f).  x spacing is passed in the separable form MasterGrid.f
 * builds it: s1(i,j) = row_scale(j) * dx(i). */
typedef struct cliffs_grid_desc {
  int32_t nx, ny;          /* nXn, nYn; at least one must exceed 2 */
  const double *dep;       /* (nx,ny) depth, >0 water, after wall/deformation */
  const double *dx;        /* (nx-1) x-spacing factor; may be NULL if nx <= 2 */
  const double *row_scale; /* (ny) cos(lat) factor, NULL for all ones */
  const double *dy;        /* (ny-1) s2; may be NULL if ny <= 2 */
  const double *zeta;      /* (ny) metric term or channel width; NULL = 0 */
  double ground;           /* minimal flow depth (allabout.f:44) */
  double crough;           /* Manning n**2 (allabout.f:46) */
  double dt;               /* time step (allabout.f:55) */
} cliffs_grid_desc;

/* Interpolation tables of one nested child grid, as NestedGrid.f:104-119
 * builds them with pinpoint (NestedGrid.f:129-148).  Indices 1-based. */
typedef struct cliffs_nest_desc {
  int32_t mm, nn;               /* child nXnst, nYnst */
  int32_t W_nx, E_nx, S_ny, N_ny;
  double W_cx, E_cx, S_cy, N_cy;
  const int32_t *WE_ny;         /* (nn) */
  const double *WE_cy;          /* (nn) */
  const int32_t *SN_nx;         /* (mm) */
  const double *SN_cx;          /* (mm) */
} cliffs_nest_desc;

/* Derived runup measures over the max-wave fields. */
typedef struct cliffs_runup {
  double max_runup;      /* max(-dep) over land cells (dep<0) ever wetted */
  int32_t i, j;          /* 1-based node of max_runup (0 if none) */
  int64_t wetted_land;   /* land cells ever wetted */
  int64_t wet_now;       /* cells currently wet */
} cliffs_runup;

/* MasterGrid.f:85-116 restated: the spacing factors of cliffs_grid_desc from
 * grid coordinates.  Replaces the s1/s2/zeta computation of MasterGrid; the
 * optional zeta override of MasterGrid.f:118-121 (channel width) is the
 * caller's.  Outputs may be NULL when the grid shape does not use them. */
int cliffs_gpu_metrics(int32_t nx, int32_t ny, int32_t cartesian,
                       const double *xcrd, const double *ycrd, double *dx,
                       double *row_scale, double *dy, double *zeta);

/* Allocate device state for one grid (replaces the allocate() calls of
 * cliffs_main.f:191-197 and 288).  hmax/velmax start at zero and edges at
 * still water, as in the reference.  CLIFFS_ERR_ARG for a grid past the
 * launch limits: ny <= 65535 when the grid has an x-sweep (nx > 2), and
 * ny <= 1,048,560 otherwise. */
int cliffs_gpu_create(const cliffs_grid_desc *desc, cliffs_ctx **out);
void cliffs_gpu_destroy(cliffs_ctx *ctx);

/* Use the caller's cudaStream_t (passed as void*) instead of the context's
 * own stream.  NULL restores the context stream. */
int cliffs_gpu_set_stream(cliffs_ctx *ctx, void *stream);

/* Initial state from total depth H = cel after apply_initial_conditions
 * (before the celerity transform of cliffs_main.f:218-227, which this call
 * applies) and velocities xvel, yvel (NULL = 0).  Resets hmax/velmax. */
int cliffs_gpu_set_initial(cliffs_ctx *ctx, const double *H,
                           const double *xvel, const double *yvel);

/* State in the reference's own form: celerity cel (= sqrt(g*H)), xvel, yvel
 * (module MASTER).  Upload does not touch hmax/velmax.
 * Transfers (set_initial, upload_state, download_state, get_maxwave): when
 * every array of the call is pinned host memory (cliffs_gpu_host_alloc,
 * cudaHostAlloc, cudaHostRegister), the conversion kernel reads or writes it
 * in place; pageable arrays go through a device staging area and the copy
 * engines.  The results are the same; every transfer synchronises. */
int cliffs_gpu_upload_state(cliffs_ctx *ctx, const double *cel,
                            const double *xvel, const double *yvel);
int cliffs_gpu_download_state(cliffs_ctx *ctx, double *cel, double *xvel,
                              double *yvel);

/* Analytic source (no reference counterpart; the reference reads a deformation
 * lattice and interpolates it, apply_initial_conditions.f, which the driver
 * keeps).  Uplift q(x,y) = amp * (exp(-(a^2+b^2)) - dipole * exp(-(a^2+b2^2)))
 * with (a, b) the offset from (x0, y0) in the source's own axes (first axis
 * rotated by angle from +x, counter-clockwise) divided by (ax, ay), and b2 =
 * b + 2 (a trough two half-widths along the second axis).  Coordinates are
 * the grid's (metres, or degrees on a spherical grid). */
typedef struct cliffs_source {
  double x0, y0;     /* centre */
  double ax, ay;     /* e-folding half-widths along the source's axes (> 0) */
  double angle;      /* radians, counter-clockwise from +x */
  double amp;        /* peak uplift (m) */
  double dipole;     /* trough depth as a fraction of amp (0: none) */
  double rise_time;  /* s: the surface uplift grows linearly over this time,
                        applied by cliffs_gpu_step; 0: at once */
  int32_t bottom;    /* 1: the bottom moves under the water column
                        (cliffs_main.f:205-208, quake = 1; rise_time must be
                        0); 0: the surface moves (209-213) */
} cliffs_source;
/* Evaluate the source on the device (FP64) and apply it to the current state;
 * xcrd (nx), ycrd (ny) are the grid coordinates. */
int cliffs_gpu_add_source(cliffs_ctx *ctx, const double *xcrd, const double *ycrd,
                          const cliffs_source *src);

/* apply_initial_conditions.f:7-70 on the device.  A lattice of nxq x nyq
 * values q (x fastest) at ascending coordinates xq (nxq), yq (nyq) is
 * interpolated bilinearly onto the grid nodes xcrd (nx), ycrd (ny) that lie
 * within it, and the result is added to the target field.  A lattice one
 * node wide along an axis interpolates along the other axis only; one two
 * nodes wide, or narrower along both axes, changes nothing.  Targets:
 * - SURFACE: the water column, as the initial surface deformation of
 *   cliffs_main.f:209-213.  A dry node floods once its depth exceeds ground.
 * - BOTTOM: the bottom rises by q under the water column (quake = 1,
 *   cliffs_main.f:205-208).
 * - XVEL, YVEL: the velocity components (get_initial_state.f's uinput,
 *   vinput).
 * Call after cliffs_gpu_set_initial; synchronises. */
enum { CLIFFS_LATTICE_SURFACE = 0, CLIFFS_LATTICE_BOTTOM = 1, CLIFFS_LATTICE_XVEL = 2, CLIFFS_LATTICE_YVEL = 3 };
int cliffs_gpu_apply_lattice(cliffs_ctx *ctx, const double *xcrd, const double *ycrd,
                             int32_t nxq, int32_t nyq, const double *xq, const double *yq,
                             const double *q, int32_t target);

/* Boundary forcing (get_boundary_feed.f): nt records at times tinput(nt);
 * west/east (ny,3,nt) and south/north (nx,3,nt) hold (u, v, eta) per edge
 * node, either pair may be NULL when that sweep does not run.  irec is the
 * 1-based start record (get_boundary_feed.f:144-167), freeze the stop flag of
 * allabout.f:65.  The time-loop cursor of cliffs_main.f:305-315 is kept by the
 * library.  nt = 0 removes the forcing. */
int cliffs_gpu_set_feed(cliffs_ctx *ctx, int32_t nt, const double *tinput,
                        const double *west, const double *east,
                        const double *south, const double *north,
                        int32_t irec, int32_t freeze);
/* First record whose edge elevation reaches cuke (get_boundary_feed.f:144-167);
 * -1 when the signal stays below it.  Uses the records of cliffs_gpu_set_feed. */
int cliffs_gpu_feed_start(cliffs_ctx *ctx, double cuke);

/* Advance nsteps time steps (cliffs_main.f:304-355): t += dt, forcing record
 * and edge interpolation, x-sweep over rows 2..ny-1 (or row 1 in 1-D),
 * y-sweep over columns 2..nx-1 (or column 1), max-wave update.  *t is the
 * model time (tinput(irec) at start).  Returns CLIFFS_FEED_ENDED with
 * *steps_done < nsteps when the forcing ended and freeze is set.  Does not
 * synchronise the stream.
 * The max-wave fields hold every completed step's end state, as the
 * reference's update after each step leaves them, whenever they are read
 * (get_maxwave, get_max_raw, runup).  In a two-dimensional grid the tiled
 * kernels fold a step's end state in during the next step's x-sweep, and
 * the readers fold the latest one in first. */
int cliffs_gpu_step(cliffs_ctx *ctx, int32_t nsteps, double *t,
                    int32_t *steps_done);
/* One sweep only: the OpenMP loop over call cliffs(iu, j, n) of
 * cliffs_main.f:325-329 (iu=1) or 340-344 (iu=2), with the edges currently
 * set; no max-wave update. */
int cliffs_gpu_sweep(cliffs_ctx *ctx, int32_t iu);
/* edge1/edge2 of module MASTER, (mx,3) each with mx = max(ny if the x-sweep
 * runs, nx if the y-sweep runs), as filled by cliffs_main.f:318-339; used by
 * cliffs_gpu_sweep only.  NULL clears them (still-water open boundary). */
int cliffs_gpu_set_edges(cliffs_ctx *ctx, const double *edge1,
                         const double *edge2);
/* Max-wave update alone (cliffs_main.f:347-355), with the current state:
 * for callers that step by single sweeps. */
int cliffs_gpu_maxwave_update(cliffs_ctx *ctx);

/* Output conversions (real*4 like the reference writers):
 *   maxwave   output_maxwave.f:14-27  (MaxE, MaxV; -1e32 where never wet)
 *   sea state output_sea_state.f:18-33 (subsampled eta/u/v; -1e32 where dry)
 * hmax/velmax in the reference's raw form (max celerity, max u^2+v^2). */
int cliffs_gpu_get_maxwave(cliffs_ctx *ctx, float *maxe, float *maxv);
int cliffs_gpu_get_max_raw(cliffs_ctx *ctx, double *hmax, double *velmax);
int cliffs_gpu_get_sea_state(cliffs_ctx *ctx, int32_t lonsub, int32_t latsub,
                             float *hsub, float *usub, float *vsub);
/* output_gages.f:18-29: eta (-1e32 where dry), u, v at 1-based (I,J). */
int cliffs_gpu_get_gauges(cliffs_ctx *ctx, int32_t n, const int32_t *I,
                          const int32_t *J, double *eta, double *u, double *v);
/* Runup measures from the max-wave fields (no reference counterpart). */
int cliffs_gpu_runup(cliffs_ctx *ctx, cliffs_runup *out);

/* Nested-grid feed (feed_children_grid.f:10-179).  nest_add copies the
 * child's tables to the device and returns its id. */
int cliffs_gpu_nest_add(cliffs_ctx *ctx, const cliffs_nest_desc *nest,
                        int32_t *id);
/* Arrival test and, once arrived, the (u, v, eta) records of the child's
 * west/east (nn,3) and south/north (mm,3) edges.  *arrived is the sticky
 * iarv flag (in/out).  Returns 1 when records were produced, 0 before
 * arrival. */
int cliffs_gpu_feed_child(cliffs_ctx *ctx, int32_t id, double cuke,
                          int32_t *arrived, double *uvq_w, double *uvq_e,
                          double *uvq_s, double *uvq_n);

/* Asynchronous outputs (no reference counterpart: the reference writes each
 * record before it steps on).
 * - The conversion runs on the context's stream, in order with the steps.
 * - The copy to the caller's host buffers runs on a second stream behind it,
 *   overlapping the steps that follow.  No call synchronises the device.
 * - The buffers hold the record once cliffs_gpu_output_wait(ticket) has
 *   returned, or cliffs_gpu_output_done reports it.  They must stay allocated
 *   until then, and be pinned (cliffs_gpu_host_alloc) for the copy to
 *   overlap.
 * - Up to 8 outputs are in flight per context. A ninth waits on the device,
 *   not the host, for the copy of the first.
 * Per call:
 * - sea_state: as cliffs_gpu_get_sea_state.
 * - gauges: as cliffs_gpu_get_gauges, n >= 1. The indices stay on the device
 *   until a call passes others.
 * - feed_child: as cliffs_gpu_feed_child, with the arrival flag kept on the
 *   device. *arrived gets 1 when this call produced a record (the wave has
 *   reached the child), else 0 and the record buffers hold nothing. */
int cliffs_gpu_get_sea_state_async(cliffs_ctx *ctx, int32_t lonsub,
                                   int32_t latsub, float *hsub, float *usub,
                                   float *vsub, int64_t *ticket);
int cliffs_gpu_get_gauges_async(cliffs_ctx *ctx, int32_t n, const int32_t *I,
                                const int32_t *J, double *eta, double *u,
                                double *v, int64_t *ticket);
int cliffs_gpu_feed_child_async(cliffs_ctx *ctx, int32_t id, double cuke,
                                int32_t *arrived, double *uvq_w,
                                double *uvq_e, double *uvq_s, double *uvq_n,
                                int64_t *ticket);
int cliffs_gpu_output_wait(cliffs_ctx *ctx, int64_t ticket);
int cliffs_gpu_output_done(cliffs_ctx *ctx, int64_t ticket, int32_t *done);
/* Pinned host memory for the asynchronous outputs, and for transfers that
 * convert in place. */
int cliffs_gpu_host_alloc(int64_t bytes, void **p);
void cliffs_gpu_host_free(void *p);

/* Sticky status bits (CLIFFS_ST_*) since the last call; synchronises.
 * Returns CLIFFS_ERR_NAN or CLIFFS_ERR_TIMEOUT when the matching bit is set,
 * else CLIFFS_WARN_CFL when CLIFFS_ST_CFL is.
 * The Courant check has no counterpart in the reference, whose dt is fixed by
 * the user (allabout.f:55) and never checked.  Every sweep evaluates
 * (|u|+c) dt / ((dx(m-1)+dx(m))/2) along its lines on the state it reads
 * (row spacing scaled by cos(lat) on a spherical grid), reduced per warp by a
 * vote and, where a number exceeds 1, a warp max reduction; VTCS-2 is stable
 * up to 1. */
int cliffs_gpu_status(cliffs_ctx *ctx, uint32_t *flags);
/* The largest Courant number above 1 that any sweep of this context has read
 * (0 when none has); synchronises.  No counterpart in the reference. */
int cliffs_gpu_courant(cliffs_ctx *ctx, double *courant);
/* Block until queued work on the context's stream is done. */
int cliffs_gpu_sync(cliffs_ctx *ctx);

/* Kernel timing: when enabled, step() brackets every sweep (its two kernel
 * launches) with CUDA events; read returns the mean duration (ms) of x- and
 * y-sweeps and their counts since the last reset. */
int cliffs_gpu_profile(cliffs_ctx *ctx, int32_t enable);
int cliffs_gpu_profile_read(cliffs_ctx *ctx, double *x_ms, int64_t *x_count,
                            double *y_ms, int64_t *y_count);

/* Number of kernels this context has launched since it was created (every
 * entry point counts its own launches; copies and memsets are not kernels). */
int cliffs_gpu_launch_count(cliffs_ctx *ctx, int64_t *n);

/* Steps captured in one CUDA graph by cliffs_gpu_step (default 16; 0 or 1:
 * no graph).  Steps without profiling or a rising source are replayed from
 * a graph, one launch per k steps; the last steps of a call, when fewer than
 * k but at least 2, from a graph of their own length (a few such lengths are
 * kept per context).  Plain steps that find no graph of their length yet
 * run launch by launch while the graph is captured for the calls that
 * follow.  A fresh state's first step (after set_initial, an upload, a
 * source, a single sweep) runs on its own.  With boundary forcing
 * (two-dimensional grids) the graph first fills the k steps' edge tables in
 * one kernel, from the records and weights the library's cursor gives each
 * step; a chunk in which the forcing ends runs step by step. */
int cliffs_gpu_set_graph_steps(cliffs_ctx *ctx, int32_t k);
/* Capture and instantiate, without running them, the graphs that a
 * cliffs_gpu_step(ctx, nsteps) call made from the current state would
 * replay, so that the call itself only launches them (no counterpart in the
 * reference).  Graphs stay valid until the tiling, the sweep kernels or
 * graph_k change. */
int cliffs_gpu_prepare_steps(cliffs_ctx *ctx, int32_t nsteps);

/* Tuning: threads per block of the x-sweep kernel (multiple of 32, <= 256)
 * and warps per block of the y-sweep kernel (<= 8).  0 keeps the current
 * value.  Results do not depend on the tiling.  Applies to the tiled sweep
 * kernels. */
int cliffs_gpu_set_tiling(cliffs_ctx *ctx, int32_t block_x, int32_t warps_y);

/* The sweep kernels, three choices with identical results:
 * - CLIFFS_SWEEP_TILED (the default): one block per tile.  The x-sweep loads
 *   its window straight into registers; the y-sweep of a two-dimensional step
 *   has its tile (16 rows x 32 columns and a halo row each side) brought into
 *   shared memory by tensor-map copies (TMA) and stored back the same way.
 * - CLIFFS_SWEEP_DIRECT: the tiled kernels with the y-sweep's window loaded
 *   straight into registers too.
 * - CLIFFS_SWEEP_STAGED: persistent kernels, one resident grid walking the
 *   tiles.  Each block's window loads arrive in shared memory by bulk copies
 *   (TMA), one tile ahead of the compute.  On GB300 it is the slowest of the
 *   three.
 * A context whose tensor maps could not be made runs the direct kernels
 * whichever is chosen; so does a y-sweep tiling (cliffs_gpu_set_tiling) other
 * than 4 warps. */
enum { CLIFFS_SWEEP_TILED = 0, CLIFFS_SWEEP_STAGED = 1, CLIFFS_SWEEP_DIRECT = 2 };
int cliffs_gpu_set_sweep_kernel(cliffs_ctx *ctx, int32_t kind);
/* Failure-detection check of the kernels' waits for their tensor-map and
 * bulk copies: one staged x-sweep, then (on a two-dimensional grid) one tiled
 * y-sweep, whose waits expect 16 bytes more than the copies bring, each wait
 * limited to wait_ms (1..2000); a y block waits twice before it leaves, so
 * the check takes about 2 * wait_ms per wave of y blocks.  Expected result:
 * CLIFFS_ERR_TIMEOUT, read by the host, when both sweeps reported their
 * waits running out, with the device usable afterwards.  The state is
 * unchanged: the sweeps write the other state copy, which is not taken.
 * CLIFFS_ERR_STATE without a state, an x-sweep or the staged kernels. */
int cliffs_gpu_check_stage_timeout(cliffs_ctx *ctx, int32_t wait_ms);

/* One sweep without any device allocation, for callers that cannot allocate
 * device memory: an application that gives the solver a fixed memory budget
 * and forbids cudaMalloc afterwards, or a time loop that must not pay the
 * implicit device synchronisation of cudaMalloc.  This entry point has no
 * counterpart in the reference; it is the x-sweep (iu=1) or y-sweep (iu=2)
 * of cliffs_gpu_sweep on arrays the caller owns.
 *
 * Arrays are device FP32 in the library's own state form: dep (depth, >0
 * water), srf (surface state: the elevation eta = H - dep where dep >= 0, the
 * water depth H where dep < 0; a drying cell keeps H = c|c|/g), xvel, yvel,
 * ny rows of `pitch` floats (pitch >= nx, a multiple of 4, every
 * pointer 16-byte aligned).  Output rows are written whole, so columns
 * nx..pitch-1 of the outputs may change.  The grid is Cartesian with uniform
 * spacing dx (x-sweep) or dy (y-sweep), still-water open edges, no max-wave.
 * Rows (iu=1) 2..ny-1 or columns (iu=2) 2..nx-1 are swept (row/column 1 on a
 * 1-D grid); the other lines are copied.  The work is queued on `stream`
 * (NULL: the default stream); nothing is synchronised.
 *
 * Limit: nx*ny <= 1048576 cells (CLIFFS_ERR_ARG beyond).  The scratch is a
 * fixed 4 MiB device array inside the library that every GPU loading it keeps
 * until the process exits; all calls share it, so calls that overlap on the
 * GPU (different streams, or devices sharing a process without ordering) race
 * on it.  The first call on each device looks up the array's device address
 * (cudaGetSymbolAddress); make that first call before any stream capture.
 * Host threads that make their first calls at the same time are serialised
 * by a lock around that look-up.  Each call clears the shared status word
 * and the worklist counter before its kernels run. */
int cliffs_gpu_sweep_noalloc(int32_t iu, int32_t nx, int32_t ny, int32_t pitch,
                             const float *dep, const float *srf,
                             const float *xvel, const float *yvel,
                             float *srf_out, float *xvel_out, float *yvel_out,
                             double dx, double dy, double ground, double crough,
                             double dt, void *stream);
/* Status of the latest cliffs_gpu_sweep_noalloc call on this device, read
 * after `stream` (the call's stream) has finished: *flags gets its
 * CLIFFS_ST_* bits (CLIFFS_ST_NAN when the sweep produced a non-finite
 * value), *listed the number of cells the sweep sent through the full
 * wet/dry rules (shorelines, line ends, supercritical windows).  Either
 * pointer may be NULL.  Synchronises the stream and allocates nothing.
 * Returns CLIFFS_ERR_NAN when CLIFFS_ST_NAN is set.  No counterpart in the
 * reference. */
int cliffs_gpu_sweep_noalloc_status(void *stream, uint32_t *flags, uint32_t *listed);

/* ---- ensembles ------------------------------------------------------------
 * No reference counterpart: the reference runs one grid per process.  A batch
 * steps many independent contexts (one source scenario each, grids of any
 * size) together: every scenario's sweeps are cut into the single-grid
 * kernels' tiles, the tiles of all scenarios form one list per sweep
 * direction, and either one cooperative launch covers many steps (blocks meet
 * at a grid barrier between the x and y phases) or one launch per phase and
 * step covers every scenario, replayed from a CUDA graph.  Results are
 * bit-identical to stepping the contexts one by one with cliffs_gpu_step.
 * Contexts must be 2-D, hold a state, have no boundary forcing, and live on
 * the current device; a source still rising (cliffs_gpu_add_source) is
 * stepped through its rise one step at a time before the plan takes over; their own entry points (gauges, max-wave, runup,
 * download) stay usable between batch steps.  The caller keeps each
 * context's model time (t += nsteps * dt). */
typedef struct cliffs_batch cliffs_batch;
enum { CLIFFS_BATCH_PERSISTENT = 0, CLIFFS_BATCH_GRAPH = 1 };
typedef struct cliffs_batch_plan {
  int32_t mode;         /* CLIFFS_BATCH_PERSISTENT or CLIFFS_BATCH_GRAPH */
  int32_t ctas_per_sm;  /* persistent: resident blocks per SM of the launch */
  int32_t graph_steps;  /* graph: steps captured in one CUDA graph; the last
                           steps of a call, when fewer (at least 2), replay
                           from a graph of their own length */
  int32_t x_rows;       /* tile shape, x phases: rows of one 512-cell column
                           chunk per tile (1..64; 0 = 1) */
  int32_t y_groups;     /* tile shape, y phases: 16-row groups of one
                           32-column group per tile (1..64; 0 = 1) */
} cliffs_batch_plan;

int cliffs_batch_create(cliffs_ctx *const *ctxs, int32_t n, cliffs_batch **out);
void cliffs_batch_destroy(cliffs_batch *b);
int cliffs_batch_set_plan(cliffs_batch *b, const cliffs_batch_plan *plan);
int cliffs_batch_get_plan(const cliffs_batch *b, cliffs_batch_plan *plan);
/* Advance every context nsteps steps; synchronises at the end.  Returns
 * CLIFFS_ERR_TIMEOUT if a grid barrier wait ran out: some blocks may then
 * have written later phases than others, so every context's state is
 * undefined (a mix of steps, its step count not advanced) until the caller
 * uploads a state again (cliffs_gpu_upload_state). */
int cliffs_batch_step(cliffs_batch *b, int32_t nsteps);
/* Time the candidate plans from a snapshot of the state, restore the
 * snapshot and keep the fastest plan; *ms_per_step gets its time per step.
 * Candidates: persistent with 1..max resident blocks per SM (tile shapes
 * 1x1 and 2x2), and graphs of 8 and 32 steps with x_rows and y_groups each
 * in {1, 2, 4}.  A persistent plan is timed over probe_steps steps after one
 * warm-up step; a graph plan over whole replays of its graph (at least
 * probe_steps steps) after one replay that builds it. */
int cliffs_batch_autotune(cliffs_batch *b, int32_t probe_steps, double *ms_per_step);
/* Failure-detection check of the grid barrier: one persistent launch whose
 * first barrier waits for an arrival that no block makes, with the wait
 * limited to wait_ms (1..2000).  Then, when the batch's y phase runs on
 * tiles by tensor-map copies, one such phase whose copy waits expect 16
 * bytes more than the copies bring (each block waits twice, about
 * 2 * wait_ms per wave of blocks).  Expected result: CLIFFS_ERR_TIMEOUT
 * (both reported), read by the host, with the device usable afterwards.
 * The persistent launch applies the x-sweep of one step to the contexts
 * before the barrier: their state is undefined until uploaded again. */
int cliffs_batch_check_barrier_timeout(cliffs_batch *b, int32_t wait_ms);
/* Gauges of every scenario, sampled in one launch (output_gages.f:18-29 for
 * all contexts of the batch).  set_gauges takes counts[n] (gauges per
 * scenario, in the batch's context order) and the 1-based nodes I, J of all
 * scenarios concatenated; get_gauges fills eta (-1e32 where dry), u, v in
 * the same order, from the state after the last batch step, and
 * synchronises. */
int cliffs_batch_set_gauges(cliffs_batch *b, const int32_t *counts, const int32_t *I, const int32_t *J);
int cliffs_batch_get_gauges(cliffs_batch *b, double *eta, double *u, double *v);
/* Kernels the batch has launched (a persistent launch counts once). */
int cliffs_batch_launch_count(const cliffs_batch *b, int64_t *n);

/* Offline tool: depth_ssl (depth_ssl/depth_ssl.f:222-362, setSSLim) on the
 * device.  It limits depth ratios between neighbouring nodes, for the
 * stability of VTCS-2.  dep (nx*ny, x fastest, FP64, > 0 water) is changed in
 * place.  Two phases, each of up to 12 passages along every column and then
 * every row:
 * - open water: a node whose sqrt(depth) differs from a neighbour's by more
 *   than the ratio alpha, with all three nodes at least depmin deep, takes
 *   the mean of its neighbours' sqrt(depth);
 * - coastlines: a wet node with land on exactly one side is made at least
 *   (its wet neighbour's depth) / alpha^2 deep.
 * The reference's defaults are alpha = 2, depmin = 0.1 m; its interactive
 * bounds are 1.5 <= alpha <= 2.5.  counts[24] gets the nodes adjusted per
 * passage (open water, then coastlines; 0 after a phase's last).
 * *status = bit 0 / bit 1 when a phase was still adjusting at its 12th
 * passage (the reference's "processing is not complete").  Results are
 * bit-identical to the sequential FP64 scan. */
int cliffs_depth_ssl(int32_t nx, int32_t ny, double *dep, double alpha, double depmin,
                     int32_t *counts, int32_t *status);

/* Offline tool: ComputeBoundaryInput (cmpboundary/cmpboundary.f:44-190) on
 * the device.  It builds the edge forcing records of a target grid
 * (get_boundary_feed.f's input) from a coarse sea-state cube.  The caller
 * cuts the cube to the target's footprint in the source lattice: columns
 * W_nx .. E_nx+1, rows S_ny .. N_ny+1 of the tables (cliffs_nest_desc, with
 * pinpoint of the target's coordinates in the source's), x fastest, then
 * rows, then records.  Values below -1e10 count as missing (0).
 * - scan (scan4wave.f): *first gets the first 1-based record whose largest
 *   value or largest negated value exceeds cuke, or nt + 1 when none does.
 *   As in the reference, *first >= nt counts as no signal (a first signal
 *   at the last record included); the caller decides what follows.
 * - edges (InterpolateOntoBndr.f:6-38): component ival (1 u, 2 v, 3 eta) of
 *   the records west/east (nn,3,nt) and south/north (mm,3,nt), Fortran order.
 *   Each value is first linear across the edge, between the lattice columns
 *   (rows) that straddle it, then linear along the edge.  Values are taken
 *   times scale first, as a single-precision product (1 for metres, 0.01
 *   for centimetres, get_sea_state.f).  The other components are left as
 *   passed.
 * Results are bit-identical to the sequential FP64 computation. */
int cliffs_boundary_scan(int32_t nx, int32_t ny, int32_t nt, const float *cube, double cuke,
                         int32_t *first);
int cliffs_boundary_edges(const cliffs_nest_desc *tables, int32_t nx, int32_t ny, int32_t nt,
                          const float *cube, double scale, int32_t ival, double *west,
                          double *east, double *south, double *north);

const char *cliffs_gpu_strerror(int code);

#ifdef __cplusplus
}
#endif
#endif
