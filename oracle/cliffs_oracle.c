/*
 * cliffs_oracle.c -- FP64 CPU restatement of the Cliffs hot path.
 *
 * TEST INFRASTRUCTURE ONLY (see cliffs_oracle.h): the checker for the CUDA
 * library and the timed CPU baseline.  The line update (orc_line) is pinned
 * bit for bit to the reference's own subroutine cliffs (cliffs.f:17-346),
 * translated from the checkout's Fortran and compiled by oracle/ref_f2c.py;
 * the whole restatement is pinned at physics level against the analytic
 * runup profiles shipped in Examples/slpbeach.zip.
 *
 * Every function names the reference lines it follows.  Expressions keep the
 * reference's operand order; build with -ffp-contract=off so that no fused
 * multiply-add changes the rounding between x86 and Arm hosts.
 */
#include "cliffs_oracle.h"

#include <stdlib.h>
#include <tgmath.h> /* sqrt, fabs, ... of the argument's type: float in the FP32 variant */
#undef I            /* complex.h's imaginary unit, which tgmath.h brings in */
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define IX(i, j, nx) ((size_t)((i) - 1) + (size_t)((j) - 1) * (size_t)(nx))

/* Automatic arrays of subroutine cliffs (cliffs.f:24-33), 1-based. */
typedef struct {
  int cap;
  orc_real *h, *pp, *qq, *vv, *dx, *scl, *depth, *Pinv, *Qinv, *v, *u;
  orc_real *hf, *uf, *vf; /* flood-modified copies, local-rule variant */
  int *lghost, *rghost;
  unsigned char *land, *newland, *R, *L;
  orc_real *pqvdL, *pqvdR; /* (4, cap) */
} line_scratch;

static int scratch_init(line_scratch *s, int n) {
  memset(s, 0, sizeof(*s));
  s->cap = n + 2;
  const size_t m = (size_t)s->cap;
  orc_real **d[] = {&s->h,    &s->pp,   &s->qq, &s->vv, &s->dx, &s->scl,
                  &s->depth, &s->Pinv, &s->Qinv, &s->v, &s->u, &s->hf,
                  &s->uf,   &s->vf};
  for (size_t k = 0; k < sizeof(d) / sizeof(d[0]); ++k) {
    *d[k] = (orc_real *)calloc(m, sizeof(orc_real));
    if (!*d[k]) return -1;
  }
  s->lghost = (int *)calloc(m, sizeof(int));
  s->rghost = (int *)calloc(m, sizeof(int));
  s->land = (unsigned char *)calloc(m, 1);
  s->newland = (unsigned char *)calloc(m, 1);
  s->R = (unsigned char *)calloc(m, 1);
  s->L = (unsigned char *)calloc(m, 1);
  /* The reference dimensions pqvdL/pqvdR(4,99) and writes them at index kseg
   * without a bound (cliffs.f:26).  The oracle sizes them by the line length
   * and reports kseg > 99 through orc_grid.seg_overflow instead. */
  s->pqvdL = (orc_real *)calloc(4 * m, sizeof(orc_real));
  s->pqvdR = (orc_real *)calloc(4 * m, sizeof(orc_real));
  if (!s->lghost || !s->rghost || !s->land || !s->newland || !s->R || !s->L ||
      !s->pqvdL || !s->pqvdR)
    return -1;
  return 0;
}

static void scratch_free(line_scratch *s) {
  orc_real *d[] = {s->h,    s->pp,   s->qq,   s->vv, s->dx, s->scl, s->depth,
                 s->Pinv, s->Qinv, s->v,    s->u,  s->hf, s->uf,  s->vf};
  for (size_t k = 0; k < sizeof(d) / sizeof(d[0]); ++k) free(d[k]);
  free(s->lghost);
  free(s->rghost);
  free(s->land);
  free(s->newland);
  free(s->R);
  free(s->L);
  free(s->pqvdL);
  free(s->pqvdR);
}

#define PQ(a, r, k) ((a)[(size_t)((r) - 1) + 4 * (size_t)(k)])

/* cliffs.f:36-54: gather line irw into the automatic arrays. */
static int gather(const orc_grid *g, int iu, int irw, line_scratch *s) {
  const int nx = g->nx;
  int n;
  if (iu == 1) {
    n = g->nx;
    for (int i = 1; i <= n; ++i) {
      s->depth[i] = g->dep[IX(i, irw, nx)];
      s->h[i] = g->cel[IX(i, irw, nx)];
      s->u[i] = g->xvel[IX(i, irw, nx)];
      s->v[i] = g->yvel[IX(i, irw, nx)];
      s->scl[i] = 0;
    }
    for (int i = 1; i <= n - 1; ++i) s->dx[i] = g->s1[IX(i, irw, nx - 1)];
  } else {
    n = g->ny;
    for (int i = 1; i <= n; ++i) {
      s->depth[i] = g->dep[IX(irw, i, nx)];
      s->h[i] = g->cel[IX(irw, i, nx)];
      s->u[i] = g->yvel[IX(irw, i, nx)];
      s->v[i] = g->xvel[IX(irw, i, nx)];
      s->scl[i] = g->zeta ? g->zeta[i - 1] : 0.0;
    }
    for (int i = 1; i <= n - 1; ++i) s->dx[i] = g->s2[i - 1];
  }
  return n;
}

/* cliffs.f:331-343: scatter back. */
static void scatter(orc_grid *g, int iu, int irw, int n, const line_scratch *s) {
  const int nx = g->nx;
  if (iu == 1) {
    for (int i = 1; i <= n; ++i) {
      g->cel[IX(i, irw, nx)] = s->h[i];
      g->xvel[IX(i, irw, nx)] = s->u[i];
      g->yvel[IX(i, irw, nx)] = s->vv[i];
    }
  } else {
    for (int i = 1; i <= n; ++i) {
      g->cel[IX(irw, i, nx)] = s->h[i];
      g->xvel[IX(irw, i, nx)] = s->vv[i];
      g->yvel[IX(irw, i, nx)] = s->u[i];
    }
  }
}

/* cliffs.f:175-251: VTCS-2 update of interior cell i given its left (1) and
 * right (2) neighbour states.  Writes pp(i), qq(i), vv(i). */
static inline void vtcs2_cell(const orc_grid *g, line_scratch *s, int i,
                              orc_real p1, orc_real q1, orc_real v1, orc_real d1,
                              orc_real p2, orc_real q2, orc_real v2, orc_real d2) {
  const orc_real grav = ORC_GRAV;
  const orc_real ground = g->ground, crough = g->crough, dt = g->dt;
  orc_real uj = s->u[i];
  orc_real vj = s->v[i];
  orc_real hj = s->h[i] * s->h[i] / grav;
  /* Almost Manning (cliffs.f:204) */
  orc_real cc = grav * crough * uj * sqrt((uj * uj + vj * vj) / hj) / hj;
  orc_real pj = s->Pinv[i];
  orc_real qj = s->Qinv[i];
  orc_real sphr = (pj - qj) * (pj + qj) * s->scl[i];
  orc_real fm = s->dx[i - 1];
  orc_real fp = s->dx[i];
  orc_real dtx = dt / (fm + fp);
  orc_real dj = s->depth[i];
  orc_real dpj = grav * (d2 - dj);
  orc_real dpm = grav * (dj - d1);
  int water = (dj > ground) && (d1 > ground) && (d2 > ground);
  orc_real ej, e2, e1, Qpj, Qjm, Qsum;

  ej = 3 * pj + qj;
  e2 = 3 * p2 + q2;
  e1 = 3 * p1 + q1;
  Qpj = (0.125 * (e2 + ej) * (p2 - pj) - dpj) / fp;
  Qjm = (0.125 * (ej + e1) * (pj - p1) - dpm) / fm;
  if ((e1 < 0) && (e2 > 0) && water)
    Qsum = (0.25 * ej * (p2 - p1) - 2 * grav * (sqrt(dj * d2) - sqrt(dj * d1))) /
           (fm + fp);
  else
    Qsum = (Qpj + Qjm) / 2;
  Qsum = Qsum + 0.25 * ej * dtx * (Qjm - Qpj);
  s->pp[i] = pj - dt * (Qsum + cc - sphr);

  ej = 3 * qj + pj;
  e2 = 3 * q2 + p2;
  e1 = 3 * q1 + p1;
  Qpj = (0.125 * (e2 + ej) * (q2 - qj) - dpj) / fp;
  Qjm = (0.125 * (ej + e1) * (qj - q1) - dpm) / fm;
  if ((e1 < 0) && (e2 > 0) && water)
    Qsum = (0.25 * ej * (q2 - q1) - 2 * grav * (sqrt(dj * d2) - sqrt(dj * d1))) /
           (fm + fp);
  else
    Qsum = (Qpj + Qjm) / 2;
  Qsum = Qsum + 0.25 * ej * dtx * (Qjm - Qpj);
  s->qq[i] = qj - dt * (Qsum + cc + sphr);

  Qsum = (v2 - vj) / fp - (vj - v1) / fm;
  s->vv[i] = vj - uj * dtx * (v2 - v1 - Qsum * (uj * dt + fp - fm));
}

/* cliffs.f:287-329: open / forced edges. */
static void edges(const orc_grid *g, int iu, int irw, int n, line_scratch *s) {
  const orc_real grav = ORC_GRAV;
  const orc_real ground = g->ground, dt = g->dt;
  const int mx = g->mx;
  const orc_real *e1 = g->edge1, *e2 = g->edge2;
  orc_real flood = e1[(size_t)(irw - 1) + 2 * (size_t)mx] + s->depth[1];
  if (!s->newland[1] && !s->newland[2] && (flood > ground)) {
    orc_real pj = s->Pinv[1], qj = s->Qinv[1], p2 = s->Pinv[2], q2 = s->Qinv[2];
    orc_real sphr = (pj - qj) * (pj + qj) * s->scl[1];
    orc_real Qpj = (3 * (q2 + qj) + p2 + pj) * (q2 - qj) / 8 -
                 grav * (s->depth[2] - s->depth[1]);
    s->qq[1] = qj - dt * (Qpj / s->dx[1] + sphr);
    s->pp[1] = e1[(size_t)(irw - 1) + (size_t)(iu - 1) * mx] + 2 * sqrt(grav * flood);
    if (s->u[1] < 0)
      s->vv[1] = s->v[1] - dt * (s->v[2] - s->v[1]) * s->u[1] / s->dx[1];
    else
      s->vv[1] = e1[(size_t)(irw - 1) + (size_t)(2 - iu) * mx];
    s->h[1] = (s->pp[1] - s->qq[1]) / 4;
    s->u[1] = (s->pp[1] + s->qq[1]) / 2;
  }
  flood = s->depth[n] + e2[(size_t)(irw - 1) + 2 * (size_t)mx];
  if (!s->newland[n - 1] && !s->newland[n] && (flood > ground)) {
    orc_real pj = s->Pinv[n], qj = s->Qinv[n], p1 = s->Pinv[n - 1], q1 = s->Qinv[n - 1];
    orc_real sphr = (pj - qj) * (pj + qj) * s->scl[n];
    orc_real Qjm = (3 * (p1 + pj) + q1 + qj) * (pj - p1) / 8 -
                 grav * (s->depth[n] - s->depth[n - 1]);
    s->pp[n] = pj - dt * (Qjm / s->dx[n - 1] - sphr);
    s->qq[n] = e2[(size_t)(irw - 1) + (size_t)(iu - 1) * mx] - 2 * sqrt(grav * flood);
    if (s->u[n] > 0)
      s->vv[n] = s->v[n] - dt * (s->v[n] - s->v[n - 1]) * s->u[n] / s->dx[n - 1];
    else
      s->vv[n] = e2[(size_t)(irw - 1) + (size_t)(2 - iu) * mx];
    s->h[n] = (s->pp[n] - s->qq[n]) / 4;
    s->u[n] = (s->pp[n] + s->qq[n]) / 2;
  }
}

/* cliffs.f:17-346, verbatim: the serial segment scan. */
static void line_scan(orc_grid *g, int iu, int irw, line_scratch *s) {
  const orc_real grav = ORC_GRAV;
  const orc_real ground = g->ground, celmin = g->celmin;
  const orc_real sqr2 = ORC_SQR2;
  const int n = gather(g, iu, irw, s);
  orc_real *h = s->h, *u = s->u, *v = s->v, *depth = s->depth;
  int *lghost = s->lghost, *rghost = s->rghost;
  unsigned char *land = s->land, *newland = s->newland;
  int water, kseg, k1, k2, i, j, k, i1, i2;
  orc_real flood;

  for (i = 1; i <= n; ++i) {
    lghost[i] = 0;
    rghost[i] = 0;
  }
  /* Find dry areas (cliffs.f:59-63) */
  for (j = 1; j <= n; ++j) land[j] = (h[j] <= celmin);
  for (j = 1; j <= n; ++j) newland[j] = land[j];

  /* Segment scan (cliffs.f:65-111) */
  water = 0;
  kseg = 0;
  if (!land[1]) {
    water = 1;
    kseg = 1;
    lghost[1] = 1;
  }
  k1 = kseg + 1;
  for (i = 2; i <= n; ++i) {
    if (water) {
      if (land[i]) {
        flood = (h[i - 1] * h[i - 1]) / grav - depth[i - 1] + depth[i];
        if ((flood > ground) && !land[i - 1] && (u[i - 1] >= 0)) {
          u[i] = u[i - 1];
          v[i] = v[i - 1];
          h[i] = celmin;
          newland[i] = 0;
        } else {
          water = 0;
          rghost[kseg] = i;
        }
      }
    } else {
      if (!land[i]) {
        water = 1;
        kseg = kseg + 1;
        flood = (h[i] * h[i]) / grav - depth[i] + depth[i - 1];
        if ((flood > ground) && (u[i] <= 0)) {
          lghost[kseg] = (i - 2 > 1) ? i - 2 : 1;
          newland[i - 1] = 0;
          u[i - 1] = u[i];
          v[i - 1] = v[i];
          h[i - 1] = celmin;
        } else {
          lghost[kseg] = i - 1;
        }
        if (kseg > 1) {
          if (lghost[kseg] < rghost[kseg - 1]) {
            lghost[kseg] = 0;
            kseg = kseg - 1;
            rghost[kseg] = 0;
          }
        }
      }
    }
  }

  if (kseg == 0) return; /* goto 99: a fully dry line is left untouched */
  if (kseg > 99) g->seg_overflow = 1;
  if (rghost[kseg] == 0) rghost[kseg] = n;
  k2 = kseg - 1;
  if (newland[rghost[kseg]]) k2 = kseg;

  for (i = 1; i <= n; ++i)
    if (newland[i]) {
      h[i] = 0;
      u[i] = 0;
      v[i] = 0;
    }
  for (i = 1; i <= n; ++i) s->vv[i] = v[i];

  /* Riemann invariants (cliffs.f:126-164) */
  for (i = 1; i <= n; ++i) {
    s->Pinv[i] = 0;
    s->Qinv[i] = 0;
  }
  for (k = 1; k <= kseg; ++k) {
    i1 = lghost[k] + 1;
    i2 = rghost[k] - 1;
    for (i = i1; i <= i2; ++i) {
      s->Pinv[i] = u[i] + 2 * h[i];
      s->Qinv[i] = u[i] - 2 * h[i];
    }
  }
  if (k1 <= kseg)
    for (k = k1; k <= kseg; ++k) {
      j = lghost[k] + 1;
      PQ(s->pqvdL, 1, k) = -s->Qinv[j];
      PQ(s->pqvdL, 2, k) = -s->Pinv[j];
      PQ(s->pqvdL, 3, k) = v[j];
      PQ(s->pqvdL, 4, k) = depth[j];
    }
  if (k2 >= 1)
    for (k = 1; k <= k2; ++k) {
      j = rghost[k] - 1;
      PQ(s->pqvdR, 1, k) = -s->Qinv[j];
      PQ(s->pqvdR, 2, k) = -s->Pinv[j];
      PQ(s->pqvdR, 3, k) = v[j];
      PQ(s->pqvdR, 4, k) = depth[j];
    }
  if (!newland[1]) {
    s->Pinv[1] = u[1] + 2 * h[1];
    s->Qinv[1] = u[1] - 2 * h[1];
    PQ(s->pqvdL, 1, 1) = s->Pinv[1];
    PQ(s->pqvdL, 2, 1) = s->Qinv[1];
    PQ(s->pqvdL, 3, 1) = v[1];
    PQ(s->pqvdL, 4, 1) = depth[1];
  }
  if (!newland[n]) {
    s->Pinv[n] = u[n] + 2 * h[n];
    s->Qinv[n] = u[n] - 2 * h[n];
    PQ(s->pqvdR, 1, kseg) = s->Pinv[n];
    PQ(s->pqvdR, 2, kseg) = s->Qinv[n];
    PQ(s->pqvdR, 3, kseg) = v[n];
    PQ(s->pqvdR, 4, kseg) = depth[n];
  }
  for (i = 1; i <= n; ++i) {
    s->qq[i] = s->Qinv[i];
    s->pp[i] = s->Pinv[i];
  }

  /* Time-step integration (cliffs.f:169-253) */
  for (k = 1; k <= kseg; ++k) {
    i1 = lghost[k] + 1;
    i2 = rghost[k] - 1;
    if (i1 > i2) continue;
    for (i = i1; i <= i2; ++i) {
      orc_real p1, q1, v1, d1, p2, q2, v2, d2;
      if (i == i1) {
        p1 = PQ(s->pqvdL, 1, k);
        q1 = PQ(s->pqvdL, 2, k);
        v1 = PQ(s->pqvdL, 3, k);
        d1 = PQ(s->pqvdL, 4, k);
      } else {
        p1 = s->Pinv[i - 1];
        q1 = s->Qinv[i - 1];
        v1 = v[i - 1];
        d1 = depth[i - 1];
      }
      if (i == i2) {
        p2 = PQ(s->pqvdR, 1, k);
        q2 = PQ(s->pqvdR, 2, k);
        v2 = PQ(s->pqvdR, 3, k);
        d2 = PQ(s->pqvdR, 4, k);
      } else {
        p2 = s->Pinv[i + 1];
        q2 = s->Qinv[i + 1];
        v2 = v[i + 1];
        d2 = depth[i + 1];
      }
      vtcs2_cell(g, s, i, p1, q1, v1, d1, p2, q2, v2, d2);
    }
  }

  /* Recover h, u (cliffs.f:255-262) */
  for (k = 1; k <= kseg; ++k) {
    i1 = lghost[k] + 1;
    i2 = rghost[k] - 1;
    for (i = i1; i <= i2; ++i) {
      h[i] = (s->pp[i] - s->qq[i]) / 4;
      u[i] = (s->pp[i] + s->qq[i]) / 2;
    }
  }
  /* Shoreline angle limiter (cliffs.f:264-285) */
  if (k1 <= kseg)
    for (k = k1; k <= kseg; ++k) {
      i = lghost[k] + 1;
      j = i + 1;
      if (land[i]) {
        if (sqr2 * h[i] > h[j]) h[i] = h[j] / sqr2;
        if (u[i] < u[j]) u[i] = u[j];
      }
    }
  if (k2 >= 1)
    for (k = 1; k <= k2; ++k) {
      i = rghost[k] - 1;
      j = i - 1;
      if (land[i]) {
        if (sqr2 * h[i] > h[j]) h[i] = h[j] / sqr2;
        if (u[i] > u[j]) u[i] = u[j];
      }
    }

  edges(g, iu, irw, n, s);
  scatter(g, iu, irw, n, s);
}

/* The same update as line_scan with the serial scan of cliffs.f:65-122
 * replaced by per-cell rules (each decided from cells i-1..i+1):
 *   R(i) = land(i) & !land(i-1) & u(i-1) >= 0 & flood_R(i) > ground   (i>=2)
 *   L(i) = land(i) & !R(i) & !land(i+1) & u(i+1) <= 0 & flood_L(i) > ground
 *   wet-or-flooded(i) = !land(i) | R(i) | L(i)
 * Segments are the maximal runs of wet-or-flooded cells; an interior cell's
 * neighbour is the real cell when that cell is wet-or-flooded, else the mirror
 * ghost of the cell itself.  Left limiter on i iff L(i) & newland(i-1); right
 * limiter on i iff R(i) & newland(i+1).  A line with no wet cell is left
 * untouched.  The arithmetic per cell is the reference's, so results must be
 * bit-identical to line_scan; the equivalence tests check that. */
static void line_local(orc_grid *g, int iu, int irw, line_scratch *s) {
  const orc_real grav = ORC_GRAV;
  const orc_real ground = g->ground, celmin = g->celmin;
  const orc_real sqr2 = ORC_SQR2;
  const int n = gather(g, iu, irw, s);
  orc_real *h = s->h, *u = s->u, *v = s->v, *depth = s->depth;
  unsigned char *land = s->land, *ew = s->newland, *R = s->R, *L = s->L;
  int any = 0;

  for (int i = 1; i <= n; ++i) {
    land[i] = (h[i] <= celmin);
    any |= !land[i];
  }
  if (!any) return;
  for (int i = 1; i <= n; ++i) {
    R[i] = 0;
    if (i >= 2 && land[i] && !land[i - 1] && u[i - 1] >= 0) {
      orc_real flood = (h[i - 1] * h[i - 1]) / grav - depth[i - 1] + depth[i];
      R[i] = flood > ground;
    }
  }
  for (int i = 1; i <= n; ++i) {
    L[i] = 0;
    if (i <= n - 1 && land[i] && !R[i] && !land[i + 1] && u[i + 1] <= 0) {
      orc_real flood = (h[i + 1] * h[i + 1]) / grav - depth[i + 1] + depth[i];
      L[i] = flood > ground;
    }
  }
  /* flood-modified values; every copy source is a wet (unmodified) cell */
  for (int i = 1; i <= n; ++i) {
    s->hf[i] = h[i];
    s->uf[i] = u[i];
    s->vf[i] = v[i];
    if (R[i]) {
      s->hf[i] = celmin;
      s->uf[i] = u[i - 1];
      s->vf[i] = v[i - 1];
    } else if (L[i]) {
      s->hf[i] = celmin;
      s->uf[i] = u[i + 1];
      s->vf[i] = v[i + 1];
    }
  }
  for (int i = 1; i <= n; ++i) {
    ew[i] = !land[i] || R[i] || L[i];
    if (ew[i]) {
      h[i] = s->hf[i];
      u[i] = s->uf[i];
      v[i] = s->vf[i];
    } else {
      h[i] = 0;
      u[i] = 0;
      v[i] = 0;
    }
    s->vv[i] = v[i];
    s->Pinv[i] = ew[i] ? u[i] + 2 * h[i] : 0.0;
    s->Qinv[i] = ew[i] ? u[i] - 2 * h[i] : 0.0;
  }
  for (int i = 2; i <= n - 1; ++i) {
    if (!ew[i]) continue;
    orc_real p1, q1, v1, d1, p2, q2, v2, d2;
    if (ew[i - 1]) {
      p1 = s->Pinv[i - 1];
      q1 = s->Qinv[i - 1];
      v1 = v[i - 1];
      d1 = depth[i - 1];
    } else {
      p1 = -s->Qinv[i];
      q1 = -s->Pinv[i];
      v1 = v[i];
      d1 = depth[i];
    }
    if (ew[i + 1]) {
      p2 = s->Pinv[i + 1];
      q2 = s->Qinv[i + 1];
      v2 = v[i + 1];
      d2 = depth[i + 1];
    } else {
      p2 = -s->Qinv[i];
      q2 = -s->Pinv[i];
      v2 = v[i];
      d2 = depth[i];
    }
    vtcs2_cell(g, s, i, p1, q1, v1, d1, p2, q2, v2, d2);
  }
  for (int i = 2; i <= n - 1; ++i) {
    if (!ew[i]) continue;
    h[i] = (s->pp[i] - s->qq[i]) / 4;
    u[i] = (s->pp[i] + s->qq[i]) / 2;
  }
  for (int i = 2; i <= n - 1; ++i) {
    if (L[i] && !ew[i - 1]) {
      int j = i + 1;
      if (sqr2 * h[i] > h[j]) h[i] = h[j] / sqr2;
      if (u[i] < u[j]) u[i] = u[j];
    }
    if (R[i] && !ew[i + 1]) {
      int j = i - 1;
      if (sqr2 * h[i] > h[j]) h[i] = h[j] / sqr2;
      if (u[i] > u[j]) u[i] = u[j];
    }
  }
  /* edges() reads newland; here that array holds wet-or-flooded flags */
  for (int i = 1; i <= n; ++i) ew[i] = !ew[i];
  edges(g, iu, irw, n, s);
  scatter(g, iu, irw, n, s);
}

void orc_line(orc_grid *g, int iu, int irw) {
  line_scratch s;
  int n = iu == 1 ? g->nx : g->ny;
  if (scratch_init(&s, n) == 0) line_scan(g, iu, irw, &s);
  scratch_free(&s);
}

void orc_line_local(orc_grid *g, int iu, int irw) {
  line_scratch s;
  int n = iu == 1 ? g->nx : g->ny;
  if (scratch_init(&s, n) == 0) line_local(g, iu, irw, &s);
  scratch_free(&s);
}

void orc_sweep(orc_grid *g, int iu, int local) {
  const int lo = iu == 1 ? g->jj1 : g->ii1;
  const int hi = iu == 1 ? g->jj2 : g->ii2;
  const int n = iu == 1 ? g->nx : g->ny;
  int overflow = 0;
#pragma omp parallel reduction(| : overflow)
  {
    line_scratch s;
    int ok = scratch_init(&s, n) == 0;
    orc_grid gl = *g;
    gl.seg_overflow = 0;
#pragma omp for schedule(static)
    for (int j = lo; j <= hi; ++j) {
      if (!ok) continue;
      if (local)
        line_local(&gl, iu, j, &s);
      else
        line_scan(&gl, iu, j, &s);
    }
    overflow |= gl.seg_overflow;
    scratch_free(&s);
  }
  if (overflow) g->seg_overflow = 1;
}

void orc_maxwave_update(orc_grid *g) {
  const size_t n = (size_t)g->nx * (size_t)g->ny;
  for (size_t k = 0; k < n; ++k) {
    orc_real aa = g->cel[k];
    if (aa > g->hmax[k]) g->hmax[k] = aa;
    aa = g->xvel[k] * g->xvel[k] + g->yvel[k] * g->yvel[k];
    if (aa > g->velmax[k]) g->velmax[k] = aa;
  }
}

void orc_edges_lerp(orc_grid *g, const orc_feed *f, double t, int iu) {
  const int irec = f->irec; /* 1-based; tinput(irec-1) <= t < tinput(irec) */
  const double cc = (f->tinput[irec - 1] - t) / (f->tinput[irec - 1] - f->tinput[irec - 2]);
  const int len = iu == 1 ? g->ny : g->nx;
  const double *a = iu == 1 ? f->west : f->south;
  const double *b = iu == 1 ? f->east : f->north;
  const size_t rec = (size_t)len * 3;
  for (int c = 0; c < 3; ++c)
    for (int j = 0; j < len; ++j) {
      size_t o0 = (size_t)j + (size_t)c * len + (size_t)(irec - 2) * rec;
      size_t o1 = (size_t)j + (size_t)c * len + (size_t)(irec - 1) * rec;
      g->edge1[(size_t)j + (size_t)c * g->mx] = (orc_real)(a[o0] * cc + a[o1] * (1 - cc));
      g->edge2[(size_t)j + (size_t)c * g->mx] = (orc_real)(b[o0] * cc + b[o1] * (1 - cc));
    }
}

int orc_step(orc_grid *g, orc_feed *f, double *t, int istep) {
  *t = *t + g->dt;
  /* cliffs_main.f:305-315 */
  while (f && f->bndr_input && *t >= f->tinput[f->irec - 1]) {
    if (f->irec == f->nt) {
      f->bndr_input = 0;
      memset(g->edge1, 0, sizeof(orc_real) * 3 * (size_t)g->mx);
      memset(g->edge2, 0, sizeof(orc_real) * 3 * (size_t)g->mx);
      f->ended_step = istep;
      if (f->freeze) return 1;
    } else {
      f->irec = f->irec + 1;
    }
  }
  if (g->xrun) {
    if (f && f->bndr_input) orc_edges_lerp(g, f, *t, 1);
    orc_sweep(g, 1, 0);
  }
  if (g->yrun) {
    if (f && f->bndr_input) orc_edges_lerp(g, f, *t, 2);
    orc_sweep(g, 2, 0);
  }
  orc_maxwave_update(g);
  return 0;
}

int orc_run(orc_grid *g, orc_feed *f, double *t, int istep0, int nsteps) {
  for (int k = 0; k < nsteps; ++k)
    if (orc_step(g, f, t, istep0 + k)) return k;
  return nsteps;
}

void orc_wall(double *dep, int64_t n, double dwall) {
  for (int64_t k = 0; k < n; ++k)
    if (dep[k] <= dwall) dep[k] = -999;
}

orc_real orc_celerity(orc_real *cel, int64_t n, orc_real ground) {
  for (int64_t k = 0; k < n; ++k) {
    if (cel[k] <= ground)
      cel[k] = 0;
    else
      cel[k] = sqrt(ORC_GRAV * cel[k]);
  }
  return sqrt(ORC_GRAV * ground);
}

void orc_pinpoint(const double *xx, int nx, double xp, int32_t *ip, double *cp) {
  int lo = 1, hi = nx;
  while (lo + 2 <= hi) {
    int med = (lo + hi) / 2;
    if (xp > xx[med - 1])
      lo = med;
    else
      hi = med;
  }
  *ip = lo;
  if (nx > 1)
    *cp = (xx[lo] - xp) / (xx[lo] - xx[lo - 1]);
  else
    *cp = 0.5;
}

void orc_apply_ic(int nx, int ny, const double *xq, const double *yq,
                  const double *qq, int kx, int ky, const double *xp,
                  const double *yp, double *pp) {
  const double zero = (double)1.0e-21f; /* real literal 0.1e-20 */
  const double x1 = xq[0] - zero, x2 = xq[nx - 1] + zero;
  const double y1 = yq[0] - zero, y2 = yq[ny - 1] + zero;
  int32_t ii, jj;
  double xcc, ycc;
  if (nx > 2 && ny > 2) {
    for (int i = 1; i <= kx; ++i) {
      double xx = xp[i - 1];
      if (!(xx >= x1 && xx <= x2)) continue;
      orc_pinpoint(xq, nx, xx, &ii, &xcc);
      for (int j = 1; j <= ky; ++j) {
        double yy = yp[j - 1];
        if (!(yy >= y1 && yy <= y2)) continue;
        orc_pinpoint(yq, ny, yy, &jj, &ycc);
        double q = (qq[IX(ii, jj, nx)] * xcc + qq[IX(ii + 1, jj, nx)] * (1 - xcc)) * ycc +
                   (qq[IX(ii, jj + 1, nx)] * xcc + qq[IX(ii + 1, jj + 1, nx)] * (1 - xcc)) *
                       (1 - ycc);
        pp[IX(i, j, kx)] = pp[IX(i, j, kx)] + q;
      }
    }
  }
  if (ny == 1 && nx > 2) {
    for (int i = 1; i <= kx; ++i) {
      double xx = xp[i - 1];
      if (!(xx >= x1 && xx <= x2)) continue;
      orc_pinpoint(xq, nx, xx, &ii, &xcc);
      double q = qq[IX(ii, 1, nx)] * xcc + qq[IX(ii + 1, 1, nx)] * (1 - xcc);
      for (int j = 1; j <= ky; ++j) pp[IX(i, j, kx)] = pp[IX(i, j, kx)] + q;
    }
  }
  if (nx == 1 && ny > 2) {
    for (int j = 1; j <= ky; ++j) {
      double yy = yp[j - 1];
      if (!(yy >= y1 && yy <= y2)) continue;
      orc_pinpoint(yq, ny, yy, &jj, &ycc);
      double q = qq[IX(1, jj, nx)] * ycc + qq[IX(1, jj + 1, nx)] * (1 - ycc);
      for (int i = 1; i <= kx; ++i) pp[IX(i, j, kx)] = pp[IX(i, j, kx)] + q;
    }
  }
}

void orc_metrics(int nx, int ny, int cartesian, const double *xcrd,
                 const double *ycrd, double *s1, double *s2, double *zeta) {
  const double PI = ORC_PI, EarthR = ORC_EARTHR;
  const double beta = PI * EarthR / 180.;
  if (nx > 2 && s1) {
    for (int j = 1; j <= ny; ++j) {
      double alpha = cartesian ? 1.0 : cos(PI / 180. * ycrd[j - 1]);
      for (int i = 1; i <= nx - 1; ++i) {
        double r = cartesian ? xcrd[i] - xcrd[i - 1] : beta * (xcrd[i] - xcrd[i - 1]);
        s1[IX(i, j, nx - 1)] = cartesian ? r : alpha * r;
      }
    }
  }
  if (ny > 2) {
    if (cartesian) {
      if (s2)
        for (int i = 1; i <= ny - 1; ++i) s2[i - 1] = ycrd[i] - ycrd[i - 1];
      if (zeta)
        for (int i = 1; i <= ny; ++i) zeta[i - 1] = 0;
    } else {
      if (s2)
        for (int i = 1; i <= ny - 1; ++i) s2[i - 1] = beta * (ycrd[i] - ycrd[i - 1]);
      double alpha = 0.125 / EarthR;
      if (zeta)
        for (int i = 1; i <= ny; ++i) zeta[i - 1] = alpha * tan(PI / 180. * ycrd[i - 1]);
    }
  }
}

void orc_nest_tables(const double *xcrd, int nx, const double *ycrd, int ny,
                     const double *xnst, int mm, const double *ynst, int nn,
                     orc_nest *t) {
  t->mm = mm;
  t->nn = nn;
  orc_pinpoint(ycrd, ny, ynst[0], &t->S_ny, &t->S_cy);
  orc_pinpoint(ycrd, ny, ynst[nn - 1], &t->N_ny, &t->N_cy);
  for (int i = 0; i < mm; ++i) orc_pinpoint(xcrd, nx, xnst[i], &t->SN_nx[i], &t->SN_cx[i]);
  orc_pinpoint(xcrd, nx, xnst[0], &t->W_nx, &t->W_cx);
  orc_pinpoint(xcrd, nx, xnst[mm - 1], &t->E_nx, &t->E_cx);
  for (int i = 0; i < nn; ++i) orc_pinpoint(ycrd, ny, ynst[i], &t->WE_ny[i], &t->WE_cy[i]);
}

/* clm(kk,1:3) for one parent column or row, weighted by cc (feed_children_grid.f:53-73). */
static void feed_clm(const orc_grid *g, int fixed_is_col, int fixed, int a, int b,
                     double cc, double hmin, double *clm, int ld) {
  const double grav = ORC_GRAV;
  for (int k = a; k <= b; ++k) {
    size_t p = fixed_is_col ? IX(fixed, k, g->nx) : IX(k, fixed, g->nx);
    double *o = clm + (k - 1);
    if (g->dep[p] > hmin) {
      o[0] = cc * g->xvel[p];
      o[ld] = cc * g->yvel[p];
      o[2 * (size_t)ld] = cc * (g->cel[p] * g->cel[p] / grav - g->dep[p]);
    } else {
      o[0] = 0;
      o[ld] = 0;
      o[2 * (size_t)ld] = 0;
    }
  }
}

int orc_feed_child(const orc_grid *g, const orc_nest *t, double hmin,
                   double cuke, int32_t *iarv, double *uvq_w, double *uvq_e,
                   double *uvq_s, double *uvq_n) {
  const double grav = ORC_GRAV;
  const int kk1 = t->WE_ny[0], kk2 = t->WE_ny[t->nn - 1] + 1;
  const int ii1 = t->SN_nx[0], ii2 = t->SN_nx[t->mm - 1] + 1;
  const double tenth = (double)0.1f;
  if (!*iarv) {
    for (int i = ii1; i <= ii2 && !*iarv; ++i)
      for (int k = kk1; k <= kk2; ++k) {
        size_t p = IX(i, k, g->nx);
        if (g->dep[p] > hmin) {
          if (fabs(g->cel[p] * g->cel[p] / grav - g->dep[p]) > (tenth * cuke)) {
            *iarv = 1;
            break;
          }
          if ((fabs(g->xvel[p]) + fabs(g->yvel[p])) * g->cel[p] > cuke) {
            *iarv = 1;
            break;
          }
        }
      }
  }
  if (!*iarv) return 0;
  const int ld = g->nx > g->ny ? g->nx : g->ny; /* clm(nXYn,3) */
  double *clm = (double *)calloc(3 * (size_t)ld, sizeof(double));
  double *clm1 = (double *)calloc(3 * (size_t)ld, sizeof(double));
  if (!clm || !clm1) {
    free(clm);
    free(clm1);
    return -1;
  }
  /* West, East: parent column pair, then interpolation along y */
  for (int side = 0; side < 2; ++side) {
    int ii = side == 0 ? t->W_nx : t->E_nx;
    double cc = side == 0 ? t->W_cx : t->E_cx;
    double *uvq = side == 0 ? uvq_w : uvq_e;
    feed_clm(g, 1, ii, kk1, kk2, cc, hmin, clm, ld);
    feed_clm(g, 1, ii + 1, kk1, kk2, 1 - cc, hmin, clm1, ld);
    for (int c = 0; c < 3; ++c)
      for (int k = kk1; k <= kk2; ++k)
        clm[(k - 1) + (size_t)c * ld] = clm[(k - 1) + (size_t)c * ld] + clm1[(k - 1) + (size_t)c * ld];
    for (int i = 1; i <= t->nn; ++i) {
      int kk = t->WE_ny[i - 1];
      double w = t->WE_cy[i - 1];
      for (int c = 0; c < 3; ++c)
        uvq[(i - 1) + (size_t)c * t->nn] =
            clm[(kk - 1) + (size_t)c * ld] * w + clm[kk + (size_t)c * ld] * (1 - w);
    }
  }
  /* South, North: parent row pair, then interpolation along x */
  for (int side = 0; side < 2; ++side) {
    int kk = side == 0 ? t->S_ny : t->N_ny;
    double cc = side == 0 ? t->S_cy : t->N_cy;
    double *uvq = side == 0 ? uvq_s : uvq_n;
    feed_clm(g, 0, kk, ii1, ii2, cc, hmin, clm, ld);
    feed_clm(g, 0, kk + 1, ii1, ii2, 1 - cc, hmin, clm1, ld);
    for (int c = 0; c < 3; ++c)
      for (int k = ii1; k <= ii2; ++k)
        clm[(k - 1) + (size_t)c * ld] = clm[(k - 1) + (size_t)c * ld] + clm1[(k - 1) + (size_t)c * ld];
    for (int i = 1; i <= t->mm; ++i) {
      int ii = t->SN_nx[i - 1];
      double w = t->SN_cx[i - 1];
      for (int c = 0; c < 3; ++c)
        uvq[(i - 1) + (size_t)c * t->mm] =
            clm[(ii - 1) + (size_t)c * ld] * w + clm[ii + (size_t)c * ld] * (1 - w);
    }
  }
  free(clm);
  free(clm1);
  return 1;
}

int orc_feed_start(const orc_feed *f, int nx, int ny, int xrun, int yrun,
                   double cuke) {
  double w1 = 0, w2 = 0, w3 = 0, w4 = 0, wave = 0;
  int it;
  for (it = 1; it <= f->nt; ++it) {
    if (xrun) {
      const double *a = f->west + (size_t)ny * 2 + (size_t)(it - 1) * ny * 3;
      const double *b = f->east + (size_t)ny * 2 + (size_t)(it - 1) * ny * 3;
      double mxa = a[0], mna = a[0], mxb = b[0], mnb = b[0];
      for (int j = 1; j < ny; ++j) {
        if (a[j] > mxa) mxa = a[j];
        if (a[j] < mna) mna = a[j];
        if (b[j] > mxb) mxb = b[j];
        if (b[j] < mnb) mnb = b[j];
      }
      w1 = mxa > -mna ? mxa : -mna;
      w2 = mxb > -mnb ? mxb : -mnb;
    }
    if (yrun) {
      const double *a = f->south + (size_t)nx * 2 + (size_t)(it - 1) * nx * 3;
      const double *b = f->north + (size_t)nx * 2 + (size_t)(it - 1) * nx * 3;
      double mxa = a[0], mna = a[0], mxb = b[0], mnb = b[0];
      for (int i = 1; i < nx; ++i) {
        if (a[i] > mxa) mxa = a[i];
        if (a[i] < mna) mna = a[i];
        if (b[i] > mxb) mxb = b[i];
        if (b[i] < mnb) mnb = b[i];
      }
      w3 = mxa > -mna ? mxa : -mna;
      w4 = mxb > -mnb ? mxb : -mnb;
    }
    wave = w1;
    if (w2 > wave) wave = w2;
    if (w3 > wave) wave = w3;
    if (w4 > wave) wave = w4;
    if (wave >= cuke) break;
  }
  if (it >= f->nt) return -1;
  return it;
}

void orc_maxwave_out(const orc_grid *g, float *hh, float *vv) {
  const size_t n = (size_t)g->nx * (size_t)g->ny;
  for (size_t k = 0; k < n; ++k) {
    hh[k] = ORC_NAN4;
    vv[k] = ORC_NAN4;
    double aa = g->hmax[k];
    if (aa > g->celmin) {
      hh[k] = (float)((aa * aa) / ORC_GRAV - g->dep[k]);
      vv[k] = (float)sqrt(g->velmax[k]);
    }
  }
}

void orc_sea_state(const orc_grid *g, int lonsub, int latsub, float *hsub,
                   float *usub, float *vsub) {
  const int nxs = (g->nx - 1) / lonsub + 1, nys = (g->ny - 1) / latsub + 1;
  for (int j = 1; j <= nys; ++j) {
    int jj = latsub * (j - 1) + 1;
    for (int i = 1; i <= nxs; ++i) {
      int ii = lonsub * (i - 1) + 1;
      size_t p = IX(ii, jj, g->nx), o = IX(i, j, nxs);
      double aa = g->cel[p];
      if (aa > g->celmin) {
        hsub[o] = (float)((aa * aa) / ORC_GRAV - g->dep[p]);
        usub[o] = (float)g->xvel[p];
        vsub[o] = (float)g->yvel[p];
      } else {
        hsub[o] = ORC_NAN4;
        usub[o] = ORC_NAN4;
        vsub[o] = ORC_NAN4;
      }
    }
  }
}

void orc_gauges(const orc_grid *g, int n, const int32_t *I, const int32_t *J,
                double *eta, double *u, double *v) {
  for (int k = 0; k < n; ++k) {
    size_t p = IX(I[k], J[k], g->nx);
    double aa = g->cel[p];
    if (aa > g->celmin)
      eta[k] = (aa * aa) / ORC_GRAV - g->dep[p];
    else
      eta[k] = (double)ORC_NAN4;
    u[k] = g->xvel[p];
    v[k] = g->yvel[p];
  }
}

/* depth_ssl/depth_ssl.f:222-362 (setSSLim): node-wise limits on the depth
 * ratio of neighbouring nodes, for the stability of VTCS-2.  b (nx*ny, x
 * fastest) is changed in place.  Up to 12 passages of open-water smoothing:
 * along every column, then every row, a node whose celerity-like sqrt(depth)
 * differs from a neighbour's by more than the ratio alpha, with all three
 * nodes at least depmin deep, takes the mean of its neighbours' sqrt(depth)
 * (the scan runs in place along the line, so a node sees its updated left
 * neighbour).  Then up to 12 passages at coastlines: a wet node with land on
 * exactly one side is made at least (its wet neighbour's depth) / alpha^2
 * deep.  counts[0..11] and counts[12..23] get the nodes adjusted per
 * passage (0 after the last).  Returns 0, or 1 (open water) | 2 (coasts)
 * when a phase ended with nodes still adjusted in its last passage. */
int orc_depth_ssl(int nx, int ny, double *b, double alpha, double depmin, int32_t *counts) {
  const int nm = nx > ny ? nx : ny;
  double *q = (double *)malloc(sizeof(double) * (size_t)nm);
  double *p = (double *)malloc(sizeof(double) * (size_t)nm);
  int *land = (int *)malloc(sizeof(int) * (size_t)nm);
  int status = 0;
  for (int k = 0; k < 24; ++k) counts[k] = 0;
  /* one line: `len` nodes at stride `st` from b + off */
  int nodes = 0;
  for (int itry = 1; itry <= 12; ++itry) {
    nodes = 0;
    for (int dir = 0; dir < 2; ++dir) {
      const int lines = dir == 0 ? nx : ny, len = dir == 0 ? ny : nx;
      for (int L = 0; L < lines; ++L) {
        double *row = dir == 0 ? b + L : b + (size_t)L * nx;
        const size_t st = dir == 0 ? (size_t)nx : 1;
        for (int j = 0; j < len; ++j) {
          q[j] = row[j * st];
          p[j] = q[j];
          land[j] = 0;
          if (q[j] < depmin)
            land[j] = 1;
          else
            q[j] = sqrt(q[j]);
        }
        for (int j = 1; j < len - 1; ++j) {
          if (!(land[j - 1] || land[j] || land[j + 1])) {
            const double c1 = q[j + 1] / q[j];
            const double c2 = q[j - 1] / q[j];
            if (c1 > alpha || c2 > alpha) {
              q[j] = (q[j - 1] + q[j + 1]) / 2;
              p[j] = q[j] * q[j];
              nodes++;
            }
          }
        }
        for (int j = 0; j < len; ++j) row[j * st] = p[j];
      }
    }
    counts[itry - 1] = nodes;
    if (nodes == 0) break;
  }
  if (nodes != 0) status |= 1;
  const double alp2 = alpha * alpha;
  for (int itry = 1; itry <= 12; ++itry) {
    nodes = 0;
    for (int dir = 0; dir < 2; ++dir) {
      const int lines = dir == 0 ? nx : ny, len = dir == 0 ? ny : nx;
      for (int L = 0; L < lines; ++L) {
        double *row = dir == 0 ? b + L : b + (size_t)L * nx;
        const size_t st = dir == 0 ? (size_t)nx : 1;
        for (int j = 0; j < len; ++j) {
          q[j] = row[j * st];
          land[j] = q[j] < depmin;
        }
        for (int j = 1; j < len - 1; ++j) {
          if (!land[j] && ((land[j + 1] && !land[j - 1]) || (!land[j + 1] && land[j - 1]))) {
            const double dep = land[j + 1] ? q[j - 1] : q[j + 1];
            if (dep / q[j] > alp2) {
              q[j] = dep / alp2;
              nodes++;
            }
          }
        }
        for (int j = 0; j < len; ++j) row[j * st] = q[j];
      }
    }
    counts[12 + itry - 1] = nodes;
    if (nodes == 0) break;
  }
  if (nodes != 0) status |= 2;
  free(q);
  free(p);
  free(land);
  return status;
}

/* cmpboundary/scan4wave.f: the first record (1-based) of a sea-state cube
 * (nx*ny*nt, x fastest; the target footprint) with a value above cuke or
 * below -cuke, values below -1e10 counting as 0; nt + 1 when there is none
 * (the loop index after a DO loop that ran out).  The reference reports "no
 * signal above treshold" for any result >= nt. */
int orc_boundary_scan(int nx, int ny, int nt, const float *sea, double cuke) {
  const double nanum = -1.0e+10;
  int it;
  for (it = 1; it <= nt; ++it) {
    const float *s = sea + (size_t)(it - 1) * nx * ny;
    double mx = -INFINITY, mn = -INFINITY;
    for (size_t k = 0; k < (size_t)nx * ny; ++k) {
      const double v = s[k] < nanum ? 0.0 : (double)s[k];
      if (v > mx) mx = v;
      if (-v > mn) mn = -v;
    }
    if (mx > cuke) break;
    if (mn > cuke) break;
  }
  return it;
}

/* One value of the sea-state cube, 1-based (i, j, k), as get_sea_state.f
 * leaves it: below -1e10 as 0, then scaled. */
static double orc_sea_value(const float *sea, int nx, int ny, int i, int j, int k, double nanum, double scale) {
  float v = sea[(size_t)(i - 1) + (size_t)(j - 1) * nx + (size_t)(k - 1) * nx * ny];
  if (v < nanum) v = 0.0f;
  if (scale != 1.0) v = v * (float)scale; /* sea = 0.01*sea: a real*4 product */
  return (double)v;
}

/* cmpboundary/InterpolateOntoBndr.f:6-38 with get_sea_state.f: the edge
 * records of a target grid from a sea-state cube (nx*ny*nt floats, x
 * fastest, the footprint from lattice column W_nx and row S_ny), values below
 * -1e10 as 0, times scale (1 for metres, 0.01 for centimetres).  Component
 * ival (1 u, 2 v, 3 eta) of west/east (nn,3,nt) and south/north (mm,3,nt),
 * Fortran order (node fastest).  t is the nest's table (orc_nest). */
void orc_boundary_edges(const orc_nest *t, int nx, int ny, int nt, const float *sea, double scale, int ival,
                        double *west, double *east, double *south, double *north) {
  const double nanum = -1.0e+10;
#define SEA(i, j, k) orc_sea_value(sea, nx, ny, (i), (j), (k), nanum, scale)
  const int mm = t->mm, nn = t->nn;
  for (int k = 1; k <= nt; ++k) {
    for (int i = 1; i <= nn; ++i) {
      const int kk = t->WE_ny[i - 1] - t->WE_ny[0] + 1;
      const double cc = t->WE_cy[i - 1];
      const double w1 = t->W_cx * SEA(1, kk, k) + (1 - t->W_cx) * SEA(2, kk, k);
      const double w2 = t->W_cx * SEA(1, kk + 1, k) + (1 - t->W_cx) * SEA(2, kk + 1, k);
      const double e1 = t->E_cx * SEA(nx - 1, kk, k) + (1 - t->E_cx) * SEA(nx, kk, k);
      const double e2 = t->E_cx * SEA(nx - 1, kk + 1, k) + (1 - t->E_cx) * SEA(nx, kk + 1, k);
      const size_t o = (size_t)(i - 1) + (size_t)(ival - 1) * nn + (size_t)(k - 1) * 3 * nn;
      west[o] = cc * w1 + (1 - cc) * w2;
      east[o] = cc * e1 + (1 - cc) * e2;
    }
    for (int i = 1; i <= mm; ++i) {
      const int kk = t->SN_nx[i - 1] - t->SN_nx[0] + 1;
      const double cc = t->SN_cx[i - 1];
      const double s1 = t->S_cy * SEA(kk, 1, k) + (1 - t->S_cy) * SEA(kk, 2, k);
      const double s2 = t->S_cy * SEA(kk + 1, 1, k) + (1 - t->S_cy) * SEA(kk + 1, 2, k);
      const double n1 = t->N_cy * SEA(kk, ny - 1, k) + (1 - t->N_cy) * SEA(kk, ny, k);
      const double n2 = t->N_cy * SEA(kk + 1, ny - 1, k) + (1 - t->N_cy) * SEA(kk + 1, ny, k);
      const size_t o = (size_t)(i - 1) + (size_t)(ival - 1) * mm + (size_t)(k - 1) * 3 * mm;
      south[o] = cc * s1 + (1 - cc) * s2;
      north[o] = cc * n1 + (1 - cc) * n2;
    }
  }
#undef SEA
}
