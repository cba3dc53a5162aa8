/*
 * cliffs_oracle.h -- CPU restatement of the Cliffs time-stepping hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker: the parity tests,
 * smoke() and the CPU-baseline leg of bench.py call it; the product (the CUDA
 * library behind include/cliffs_gpu.h) never links or calls it.
 *
 * Parity status: the reference is Fortran (gfortran and the NetCDF libraries
 * are absent here), so it cannot be built or run.  This restatement follows
 * the reference line by line in FP64, with Fortran's default-real literals
 * rounded to float first (grav = (double)9.8f, PI = (double)3.1415926536f,
 * sqr2 = (double)1.41421356f).  It is pinned against the only known-answer
 * data the reference ships (the analytic solitary-wave runup profiles of
 * Examples/slpbeach.zip) at physics level; bit-level parity with the Fortran
 * build is UNPINNED.
 *
 * Arrays are column-major (x fastest) exactly like the Fortran module arrays:
 * element (i,j), 1-based, lives at [(i-1) + (j-1)*nx].
 *
 * The grid state and the time loop are written in orc_real: double for the
 * oracle.  The same source built with -DORC_REAL=float and
 * -fsingle-precision-constant is an FP32 variant of the CPU time loop, timed
 * beside the FP64 one as a like-for-like baseline of the FP32 GPU path; it is
 * not a checker.
 */
#ifndef CLIFFS_ORACLE_H
#define CLIFFS_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#ifndef ORC_REAL
#define ORC_REAL double
#endif
typedef ORC_REAL orc_real;

/* Fortran default-real literals widened to real*8 (global_modules.f:17, cliffs.f:34). */
#define ORC_GRAV 9.800000190734863
#define ORC_PI 3.1415927410125732
#define ORC_EARTHR 6371009.0
#define ORC_SQR2 1.4142135381698608
#define ORC_NAN4 (-1.0e32f) /* global_modules.f:18, real*4 */

/* State of module MASTER/PARAMETERS that the line solver touches
 * (global_modules.f:16-55). */
typedef struct orc_grid {
  int32_t nx, ny;
  orc_real *dep, *cel, *xvel, *yvel; /* (nx,ny) */
  orc_real *hmax, *velmax;           /* (nx,ny) */
  const orc_real *s1;                /* (nx-1,ny), NULL when nx<=2 */
  const orc_real *s2;                /* (ny-1),   NULL when ny<=2 */
  const orc_real *zeta;              /* (ny),     NULL when ny<=2 */
  orc_real ground, crough, dt, celmin;
  orc_real *edge1, *edge2; /* (mx,3) each */
  int32_t mx;
  int32_t xrun, yrun, ii1, ii2, jj1, jj2; /* cliffs_main.f:140-164 */
  int32_t seg_overflow; /* out: a line had more than 99 wet segments */
} orc_grid;

/* Boundary forcing records (get_boundary_feed.f) and the record cursor of the
 * time loop (cliffs_main.f:305-315). */
typedef struct orc_feed {
  int32_t nt;
  const double *tinput;       /* (nt) */
  const double *west, *east;  /* (ny,3,nt) */
  const double *south, *north;/* (nx,3,nt) */
  int32_t irec;               /* 1-based, as in the reference */
  int32_t bndr_input;         /* logical */
  int32_t freeze;             /* logical */
  int32_t ended_step;         /* out: step at which the feed ended, 0 if not */
} orc_feed;

/* cliffs.f:17-346 -- advance line irw along direction iu (1 = x, 2 = y). */
void orc_line(orc_grid *g, int iu, int irw);
/* Same update with the segment scan of cliffs.f:56-122 replaced by the
 * per-cell rules the GPU kernels use; used only to prove the two agree. */
void orc_line_local(orc_grid *g, int iu, int irw);
/* OpenMP loop over lines (cliffs_main.f:325-329 / 340-344).
 * local != 0 selects orc_line_local. */
void orc_sweep(orc_grid *g, int iu, int local);
/* cliffs_main.f:347-355 */
void orc_maxwave_update(orc_grid *g);
/* cliffs_main.f:318-324 (iu=1) and 333-339 (iu=2). */
void orc_edges_lerp(orc_grid *g, const orc_feed *f, double t, int iu);
/* One pass of the time loop body cliffs_main.f:304-355 (no file output).
 * Returns 1 when the feed ended with freeze set (the reference jumps to its
 * final output), else 0. */
int orc_step(orc_grid *g, orc_feed *f, double *t, int istep);
/* nsteps passes of orc_step starting at step istep0; returns the number of
 * steps completed. */
int orc_run(orc_grid *g, orc_feed *f, double *t, int istep0, int nsteps);

/* cliffs_main.f:131-137 */
void orc_wall(double *dep, int64_t n, double dwall);
/* cliffs_main.f:218-227: cel <- 0 if cel<=ground else sqrt(grav*cel);
 * returns celmin = sqrt(grav*ground). */
orc_real orc_celerity(orc_real *cel, int64_t n, orc_real ground);
/* apply_initial_conditions.f:7-70 */
void orc_apply_ic(int nx, int ny, const double *xq, const double *yq,
                  const double *qq, int kx, int ky, const double *xp,
                  const double *yp, double *pp);
/* NestedGrid.f:129-148 (ip is 1-based). */
void orc_pinpoint(const double *xx, int nx, double xp, int32_t *ip, double *cp);
/* MasterGrid.f:85-116: s1 (nx-1,ny), s2 (ny-1), zeta (ny).  Pass NULL for
 * outputs that the grid shape does not allocate. */
void orc_metrics(int nx, int ny, int cartesian, const double *xcrd,
                 const double *ycrd, double *s1, double *s2, double *zeta);

/* Interpolation tables for one nested grid (NestedGrid.f:104-119). */
typedef struct orc_nest {
  int32_t mm, nn;           /* child nXnst, nYnst */
  int32_t W_nx, E_nx, S_ny, N_ny;
  double W_cx, E_cx, S_cy, N_cy;
  int32_t *WE_ny; double *WE_cy; /* (nn) */
  int32_t *SN_nx; double *SN_cx; /* (mm) */
} orc_nest;
void orc_nest_tables(const double *xcrd, int nx, const double *ycrd, int ny,
                     const double *xnst, int mm, const double *ynst, int nn,
                     orc_nest *out);
/* feed_children_grid.f:10-179.  Updates *iarv; when the wave has arrived it
 * fills uvq_{w,e} (nn,3) and uvq_{s,n} (mm,3) column-major and returns 1,
 * else returns 0. */
int orc_feed_child(const orc_grid *g, const orc_nest *t, double hmin,
                   double cuke, int32_t *iarv, double *uvq_w, double *uvq_e,
                   double *uvq_s, double *uvq_n);
/* get_boundary_feed.f:144-167: first record whose edge |eta| >= cuke.
 * Returns the 1-based record index, or -1 when the signal stays below it. */
int orc_feed_start(const orc_feed *f, int nx, int ny, int xrun, int yrun,
                   double cuke);

/* output_maxwave.f:14-27 (real*4 results). */
void orc_maxwave_out(const orc_grid *g, float *hh, float *vv);
/* output_sea_state.f:18-33 */
void orc_sea_state(const orc_grid *g, int lonsub, int latsub, float *hsub,
                   float *usub, float *vsub);
/* output_gages.f:18-29 (I, J are 1-based). */
void orc_gauges(const orc_grid *g, int n, const int32_t *I, const int32_t *J,
                double *eta, double *u, double *v);

/* depth_ssl/depth_ssl.f:222-362 (setSSLim), in place on b (nx*ny, x fastest);
 * counts[24]: nodes adjusted per passage, open water then coastlines.
 * Returns 0, or 1 | 2 when a phase was still adjusting at its 12th passage. */
int orc_depth_ssl(int nx, int ny, double *b, double alpha, double depmin, int32_t *counts);

/* cmpboundary/scan4wave.f on a footprint cube (nx*ny*nt floats, x fastest):
 * the first 1-based record above cuke in magnitude, or nt + 1. */
int orc_boundary_scan(int nx, int ny, int nt, const float *sea, double cuke);
/* cmpboundary/InterpolateOntoBndr.f:6-38: component ival (1 u, 2 v, 3 eta) of
 * the edge records from the footprint cube, scaled by scale. */
void orc_boundary_edges(const orc_nest *t, int nx, int ny, int nt, const float *sea, double scale, int ival,
                        double *west, double *east, double *south, double *north);

#ifdef __cplusplus
}
#endif
#endif
