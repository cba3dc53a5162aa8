// march.cuh -- streaming VTCS-2 line update (one line per thread).
//
// Restates cliffs.f:17-346 (subroutine cliffs) for a single grid line as a
// pipeline that consumes raw cell k and emits the final value of cell k-3:
//
//   stage A (cell k)    derive H = d + eta and land = H <= ground
//   stage B (cell k-1)  flooding: R(k) and L(k-1) decide whether a dry cell is
//                       taken into the wet segment (cliffs.f:74-111); the
//                       flood-modified state of k-1 becomes final
//   stage C (cell k-2)  VTCS-2 interior update (cliffs.f:175-262) or the
//                       open/forced edge update (cliffs.f:287-329)
//   stage D (cell k-3)  shoreline angle limiter (cliffs.f:264-285) and output
//
// The serial segment scan of the reference is replaced by per-cell rules that
// depend on cells i-1..i+1 only; the oracle's orc_line_local proves them
// bit-identical to the scan in FP64.  Segments are the maximal runs of
// wet-or-flooded cells; an interior cell whose neighbour is not in its run uses
// the mirror ghost of itself (cliffs.f:137-152).  A line without any wet cell
// is left untouched (cliffs.f:113); the caller supplies that line flag.
//
// State is carried as surface elevation eta (not celerity) so that FP32 keeps
// ~1e-7 m resolution in deep water: the hydrostatic balance
// (1/8)(e2+ej)(p2-pj) - g(d2-dj) is rewritten with c^2 = g(d+eta) as
//   g(eta2-eta1) + (u1+u2)(c2-c1) + (u1+u2+c1+c2)(u2-u1)/2
// which is exact in real arithmetic and free of the catastrophic cancellation
// of the celerity form.  A negative celerity (a cell drying out) is kept as a
// negative total depth H = c|c|/g.
#pragma once

#ifdef __CUDACC__
#define CL_HD __host__ __device__ __forceinline__
#else
#define CL_HD inline
#include <cmath>
#endif

namespace cliffs {

template <typename R>
CL_HD R csqrt(R x) {
#ifdef __CUDA_ARCH__
  return sqrt(x);
#else
  return std::sqrt(x);
#endif
}

// sqrt(x) for x > 0 where ~1 ulp is enough (celerity and friction
// coefficients; the state itself is carried in eta): one MUFU op on the GPU.
CL_HD float fsqrt_pos(float x) {
#ifdef __CUDA_ARCH__
  return x * rsqrtf(x);
#else
  return std::sqrt(x);
#endif
}
CL_HD double fsqrt_pos(double x) { return csqrt(x); }

// sqrt(x) for x >= 0 (0 maps to 0).
CL_HD float fsqrt0(float x) {
#ifdef __CUDA_ARCH__
  return x * rsqrtf(fmaxf(x, 1e-30f));
#else
  return std::sqrt(x);
#endif
}
CL_HD double fsqrt0(double x) { return csqrt(x); }

// 1/sqrt(x), x > 0
CL_HD float frsqrt(float x) {
#ifdef __CUDA_ARCH__
  return rsqrtf(x);
#else
  return 1.0f / std::sqrt(x);
#endif
}
CL_HD double frsqrt(double x) { return 1.0 / csqrt(x); }

// Physical constants of one sweep (module PARAMETERS, global_modules.f:46-55).
template <typename R>
struct Phys {
  R g;        // grav = (double)9.8f
  R ginv;     // 1/g
  R ground;   // minimal flow depth
  R celmin;   // sqrt(g*ground)
  R dt;
  R idt;      // 1/dt
  R gcrough;  // g*crough
  R sqr2;     // (double)1.41421356f
};

// Geometry of cell position m along the line: fm = dx(m-1), fp = dx(m).
template <typename R>
struct Geo {
  R inv_fm, inv_fp;  // 1/fm, 1/fp
  R dtx;             // dt/(fm+fp)
  R dfpm;            // fp - fm
  R scl;             // metric term (zeta in the y-sweep, 0 in the x-sweep)
};

// One cell of the pipeline ring.
template <typename R>
struct RCell {
  R d, eta, u, v;      // raw input (u normal, v tangential)
  R H;                 // d + eta
  R c, ef, uf, vf;     // flood-modified celerity, eta, u, v
  R cn, un, vn, en;    // updated celerity, u, v, eta
  unsigned fl;         // flag bits below
};

enum : unsigned {
  F_PRESENT = 1u,  // 1 <= k <= n
  F_LAND = 2u,     // h <= celmin
  F_R = 4u,        // flooded from the left neighbour (cliffs.f:77-82)
  F_L = 8u,        // flooded from the right neighbour (cliffs.f:92-98)
  F_EW = 16u,      // wet or flooded (not newland)
};

template <typename R>
struct EdgeVals {
  R un, vt, eta;  // feed normal velocity, tangential velocity, elevation
};

template <typename R>
struct OutCell {
  R eta, u, v;  // final eta, normal and tangential velocity
};

template <typename R>
CL_HD void face_flux(R ul, R cl, R el, R ur, R cr, R er, const Phys<R>& p,
                     R& FP, R& FQ) {
  // (1/8)(e_l+e_r)(P_r-P_l) - g(d_r-d_l), e = 3P+Q = 4(u+c), and the Q analogue
  const R U = ul + ur, C = cl + cr, du = ur - ul, dc = cr - cl;
  const R gde = p.g * (er - el);
  const R Udc = U * dc;
  FP = gde + Udc + R(0.5) * (U + C) * du;
  FQ = gde - Udc + R(0.5) * (U - C) * du;
}

// H from celerity with the sign of c kept: H = c|c|/g.
template <typename R>
CL_HD R eta_from_c(R c, R d, const Phys<R>& p) {
  return c * (c < R(0) ? -c : c) * p.ginv - d;
}

// New eta after celerity c0 (with eta e0) moved by dc: exact increment form
// when both celerities are positive.
template <typename R>
CL_HD R eta_step(R c0, R e0, R dc, R d, const Phys<R>& p) {
  const R c1 = c0 + dc;
  if (c0 > R(0) && c1 > R(0)) return e0 + dc * (R(2) * c0 + dc) * p.ginv;
  return eta_from_c(c1, d, p);
}

// State of one cell as the interior update sees it (after flooding).
template <typename R>
struct CellState {
  R u, c, e, d, v, H;  // normal velocity, celerity, eta, depth, tangential, H
};

struct NoFlux {};

// VTCS-2 interior update of cell j between real neighbours a (left) and b
// (right), cliffs.f:200-262, in the eta form.  FPl/FQl, FPr/FQr are the face
// fluxes (a,j) and (j,b).  Returns the new (eta, u, v); *cn gets the new
// celerity.
template <typename R>
CL_HD OutCell<R> interior_update(const CellState<R>& a, const CellState<R>& j, const CellState<R>& b,
                                 R FPl, R FQl, R FPr, R FQr, const Geo<R>& geo, const Phys<R>& p,
                                 R* cn_out) {
  const R uj = j.u, cj = j.c, vj = j.v, dj = j.d;
  const R inv_fm = geo.inv_fm, inv_fp = geo.inv_fp, dtx = geo.dtx;
  const R r = frsqrt(j.H);  // sqrt((u^2+v^2)/H)/H = |u,v| / H^1.5 (cliffs.f:204)
  const R cc = p.gcrough * uj * fsqrt0(uj * uj + vj * vj) * (r * r * r);
  const R sphr = R(8) * cj * uj * geo.scl;  // (P-Q)(P+Q)*scl
  const R ejP = uj + cj, ejQ = uj - cj;
  const R QpP = FPr * inv_fp, QmP = FPl * inv_fm;
  const R QpQ = FQr * inv_fp, QmQ = FQl * inv_fm;
  R QsP = R(0.5) * (QpP + QmP);
  R QsQ = R(0.5) * (QpQ + QmQ);
  const bool sonP = (a.u + a.c < R(0)) && (b.u + b.c > R(0));
  const bool sonQ = (a.u - a.c < R(0)) && (b.u - b.c > R(0));
  if ((sonP || sonQ) && (dj > p.ground) && (a.d > p.ground) && (b.d > p.ground)) {
    // transcritical point (cliffs.f:228-232, 241-245)
    const R isum = dtx * p.idt;
    const R sdiff = R(2) * p.g * (csqrt(dj * b.d) - csqrt(dj * a.d));
    if (sonP) QsP = (ejP * ((b.u - a.u) + R(2) * (b.c - a.c)) - sdiff) * isum;
    if (sonQ) QsQ = (ejQ * ((b.u - a.u) - R(2) * (b.c - a.c)) - sdiff) * isum;
  }
  QsP = QsP + ejP * dtx * (QmP - QpP);
  QsQ = QsQ + ejQ * dtx * (QmQ - QpQ);
  const R dP = -p.dt * (QsP + cc - sphr);
  const R dQ = -p.dt * (QsQ + cc + sphr);
  const R Qv = (b.v - vj) * inv_fp - (vj - a.v) * inv_fm;
  OutCell<R> o;
  o.v = vj - uj * dtx * ((b.v - a.v) - Qv * (uj * p.dt + geo.dfpm));
  const R dc = R(0.25) * (dP - dQ);
  *cn_out = cj + dc;
  o.u = uj + R(0.5) * (dP + dQ);
  o.eta = eta_step(cj, j.e, dc, dj, p);
  return o;
}

// Open / forced edge update of line cell 1 (cliffs.f:288-308): C is cell 1
// and B cell 2 (flood-modified), both wet or flooded.
template <typename R>
CL_HD void edge_left(const CellState<R>& C, const CellState<R>& B, const EdgeVals<R>& e, R inv_dx1, R scl1,
                     const Phys<R>& p, R& cn, R& un, R& vn, R& en) {
  R FP, FQ;
  face_flux(C.u, C.c, C.e, B.u, B.c, B.e, p, FP, FQ);
  const R sphr = R(8) * C.c * C.u * scl1;
  const R dQ = -p.dt * (FQ * inv_dx1 + sphr);
  const R cbnd = csqrt(p.g * (C.d + e.eta));
  const R dP = (e.un - C.u) + R(2) * p.g * (e.eta - C.e) / (cbnd + C.c);
  vn = (C.u < R(0)) ? C.v - p.dt * (B.v - C.v) * C.u * inv_dx1 : e.vt;
  const R dc = R(0.25) * (dP - dQ);
  cn = C.c + dc;
  un = C.u + R(0.5) * (dP + dQ);
  en = eta_step(C.c, C.e, dc, C.d, p);
}

// Open / forced edge update of line cell n (cliffs.f:309-329): D is cell n-1,
// C cell n.
template <typename R>
CL_HD void edge_right(const CellState<R>& D, const CellState<R>& C, const EdgeVals<R>& e, R inv_dxn1, R scln,
                      const Phys<R>& p, R& cn, R& un, R& vn, R& en) {
  R FP, FQ;
  face_flux(D.u, D.c, D.e, C.u, C.c, C.e, p, FP, FQ);
  const R sphr = R(8) * C.c * C.u * scln;
  const R dP = -p.dt * (FP * inv_dxn1 - sphr);
  const R cbnd = csqrt(p.g * (C.d + e.eta));
  const R dQ = (e.un - C.u) - R(2) * p.g * (e.eta - C.e) / (cbnd + C.c);
  vn = (C.u > R(0)) ? C.v - p.dt * (C.v - D.v) * C.u * inv_dxn1 : e.vt;
  const R dc = R(0.25) * (dP - dQ);
  cn = C.c + dc;
  un = C.u + R(0.5) * (dP + dQ);
  en = eta_step(C.c, C.e, dc, C.d, p);
}

// Raw input of one line cell; present iff 1 <= position <= n.
template <typename R>
struct RawCell {
  R d, e, u, v;
  bool present;
};

// Per-line constants the wet/dry rules need.
template <typename R>
struct LineCtx {
  int n;
  bool wet;            // the line holds a wet cell (else it is left untouched)
  EdgeVals<R> eL, eR;  // forcing at cells 1 and n
  R inv_dx1, inv_dxn1, scl1, scln;
};

// Final value of line cell o from the raw cells o-3..o+3 (w[3] is cell o):
// the whole of cliffs.f:56-329 evaluated for one cell with the per-cell rules
//   R(k) = land(k) & !land(k-1) & u(k-1) >= 0 & flood from k-1  (cliffs.f:76-82)
//   L(k) = land(k) & !R(k) & !land(k+1) & u(k+1) <= 0 & flood from k+1 (89-98)
//   wet-or-flooded(k) = !land(k) | R(k) | L(k)
// an interior neighbour outside the cell's run is the mirror ghost of the cell
// (cliffs.f:137-152); the angle limiter applies to a cell flooded from the left
// (right) whose other side is newland (cliffs.f:264-285).  geo[t] is the
// geometry of positions o-1, o, o+1 (t = 0, 1, 2).
template <typename R>
CL_HD OutCell<R> general_cell(const RawCell<R> w[7], int o, const LineCtx<R>& L, const Geo<R> geo[3],
                              const Phys<R>& p) {
  bool land[7], Rf[7], Lf[7], ew[7];
  R H[7];
#pragma unroll
  for (int t = 0; t < 7; ++t) {
    H[t] = w[t].d + w[t].e;
    land[t] = !w[t].present || H[t] <= p.ground;
    Rf[t] = Lf[t] = false;
  }
#pragma unroll
  for (int t = 1; t <= 5; ++t) {
    if (w[t].present && land[t]) {
      Rf[t] = w[t - 1].present && !land[t - 1] && w[t - 1].u >= R(0) && (w[t - 1].e + w[t].d > p.ground);
      Lf[t] = !Rf[t] && w[t + 1].present && !land[t + 1] && w[t + 1].u <= R(0) &&
              (w[t + 1].e + w[t].d > p.ground);
    }
  }
  CellState<R> fm[7];
#pragma unroll
  for (int t = 0; t < 7; ++t) {
    ew[t] = w[t].present && (!land[t] || Rf[t] || Lf[t]);
    if (Rf[t] || Lf[t]) {
      const int s = Rf[t] ? t - 1 : t + 1;
      fm[t] = CellState<R>{w[s].u, p.celmin, p.ground - w[t].d, w[t].d, w[s].v, p.ground};
    } else {
      fm[t] = CellState<R>{w[t].u, fsqrt_pos(p.g * (H[t] > p.ground ? H[t] : p.ground)), w[t].e, w[t].d, w[t].v,
                           H[t]};
    }
  }
  OutCell<R> out;
  if (!ew[3]) {
    if (L.wet) {  // newland in a line with water: h=u=v=0 (cliffs.f:118-122)
      out.eta = -w[3].d;
      out.u = R(0);
      out.v = R(0);
    } else {  // a line without water is left untouched (cliffs.f:113)
      out.eta = w[3].e;
      out.u = w[3].u;
      out.v = w[3].v;
    }
    return out;
  }
  const int n = L.n;
  if (o == 1 || o == n) {
    // flood-modified value unless the edge condition holds
    out.eta = fm[3].e;
    out.u = fm[3].u;
    out.v = fm[3].v;
    R cn, un, vn, en;
    if (o == 1 && n >= 2 && ew[4] && (L.eL.eta + w[3].d > p.ground)) {
      edge_left(fm[3], fm[4], L.eL, L.inv_dx1, L.scl1, p, cn, un, vn, en);
      out.eta = en;
      out.u = un;
      out.v = vn;
    } else if (o == n && n >= 2 && ew[2] && (L.eR.eta + w[3].d > p.ground)) {
      edge_right(fm[2], fm[3], L.eR, L.inv_dxn1, L.scln, p, cn, un, vn, en);
      out.eta = en;
      out.u = un;
      out.v = vn;
    }
    return out;
  }
  // interior update of cell t with real or mirror neighbours
  auto update = [&](int t, const Geo<R>& g, R& cn) -> OutCell<R> {
    const CellState<R>& j = fm[t];
    const CellState<R> mir{-j.u, j.c, j.e, j.d, j.v, j.H};
    const CellState<R>& a = ew[t - 1] ? fm[t - 1] : mir;
    const CellState<R>& b = ew[t + 1] ? fm[t + 1] : mir;
    R FPl, FQl, FPr, FQr;
    face_flux(a.u, a.c, a.e, j.u, j.c, j.e, p, FPl, FQl);
    face_flux(j.u, j.c, j.e, b.u, b.c, b.e, p, FPr, FQr);
    return interior_update(a, j, b, FPl, FQl, FPr, FQr, g, p, &cn);
  };
  R cO;
  out = update(3, geo[1], cO);
  if (Lf[3] && !ew[2]) {
    // newly wetted cell on a left shoreline: limit against cell o+1
    R hj, uj;
    if (o + 1 <= n - 1) {
      const OutCell<R> nb = update(4, geo[2], hj);
      uj = nb.u;
    } else {
      hj = fm[4].c;
      uj = fm[4].u;
    }
    if (p.sqr2 * cO > hj) {
      cO = hj / p.sqr2;
      out.eta = eta_from_c(cO, w[3].d, p);
    }
    if (out.u < uj) out.u = uj;
  } else if (Rf[3] && !ew[4]) {
    // newly wetted cell on a right shoreline: limit against cell o-1
    R hj, uj;
    if (o - 1 >= 2) {
      const OutCell<R> nb = update(2, geo[0], hj);
      uj = nb.u;
    } else {
      hj = fm[2].c;
      uj = fm[2].u;
    }
    if (p.sqr2 * cO > hj) {
      cO = hj / p.sqr2;
      out.eta = eta_from_c(cO, w[3].d, p);
    }
    if (out.u > uj) out.u = uj;
  }
  return out;
}

template <typename R>
struct LineMarch {
  Phys<R> p;
  int n;       // line length
  bool wet;    // the line holds at least one wet cell (else untouched)
  EdgeVals<R> eL, eR;
  R inv_dx1, inv_dxn1;  // 1/dx(1), 1/dx(n-1)
  R scl1, scln;         // scl(1), scl(n)
  // ring: a = k, b = k-1, c = k-2, d = k-3, e = k-4
  RCell<R> ra, rb, rc, rd, re;
  R fpr_P, fpr_Q;  // flux at face (k-2, k-1) carried to the next update
  bool fpr_ok;

  CL_HD void init(const Phys<R>& ph, int n_, bool wet_) {
    p = ph;
    n = n_;
    wet = wet_;
    fpr_ok = false;
    RCell<R> z{};
    ra = rb = rc = rd = re = z;
  }

  // Push raw cell k (present iff 1 <= k <= n); returns true and fills `out`
  // when cell k-3 lies in [1, n].  geo_m is the geometry of m = k-2.
  CL_HD bool push(int k, R d, R eta, R u, R v, const Geo<R>& geo_m,
                  OutCell<R>& out) {
    // shift ring
    re = rd;
    rd = rc;
    rc = rb;
    rb = ra;
    RCell<R>& A = ra;  // k
    RCell<R>& B = rb;  // k-1
    RCell<R>& C = rc;  // k-2
    RCell<R>& D = rd;  // k-3
    RCell<R>& E = re;  // k-4
    // ---- stage A: cell k
    A.fl = 0;
    if (k >= 1 && k <= n) {
      A.d = d;
      A.eta = eta;
      A.u = u;
      A.v = v;
      A.H = d + eta;
      A.fl = F_PRESENT | (A.H <= p.ground ? F_LAND : 0u);
      // R(k): flooded from the wet cell k-1 moving landward (cliffs.f:76-82)
      if ((A.fl & F_LAND) && (B.fl & F_PRESENT) && !(B.fl & F_LAND) &&
          B.u >= R(0) && (B.eta + A.d > p.ground))
        A.fl |= F_R;
    }
    // ---- stage B: finalize cell k-1
    if (B.fl & F_PRESENT) {
      // L(k-1): flooded from the wet cell k moving landward (cliffs.f:89-98)
      if ((B.fl & F_LAND) && !(B.fl & F_R) && (A.fl & F_PRESENT) &&
          !(A.fl & F_LAND) && A.u <= R(0) && (A.eta + B.d > p.ground))
        B.fl |= F_L;
      if (B.fl & F_R) {
        B.c = p.celmin;
        B.ef = p.ground - B.d;
        B.uf = C.u;
        B.vf = C.v;
        B.fl |= F_EW;
      } else if (B.fl & F_L) {
        B.c = p.celmin;
        B.ef = p.ground - B.d;
        B.uf = A.u;
        B.vf = A.v;
        B.fl |= F_EW;
      } else if (!(B.fl & F_LAND)) {
        B.c = fsqrt_pos(p.g * B.H);
        B.ef = B.eta;
        B.uf = B.u;
        B.vf = B.v;
        B.fl |= F_EW;
      }
    }
    // ---- stage C: update cell m = k-2
    const int m = k - 2;
    bool carried = false;
    R carP = R(0), carQ = R(0);
    if ((C.fl & F_EW) && m >= 2 && m <= n - 1) {
      const bool lreal = (D.fl & F_EW) != 0;
      const bool rreal = (B.fl & F_EW) != 0;
      const R uj = C.uf, cj = C.c, vj = C.vf, dj = C.d;
      R FPl, FQl, FPr, FQr;
      R ua, ca, da, va, ub, cb, db, vb;
      if (lreal) {
        ua = D.uf; ca = D.c; da = D.d; va = D.vf;
        if (fpr_ok) {
          FPl = fpr_P;
          FQl = fpr_Q;
        } else {
          face_flux(ua, ca, D.ef, uj, cj, C.ef, p, FPl, FQl);
        }
      } else {  // mirror ghost of cell m (cliffs.f:137-144)
        ua = -uj; ca = cj; da = dj; va = vj;
        FPl = R(2) * cj * uj;
        FQl = -FPl;
      }
      if (rreal) {
        ub = B.uf; cb = B.c; db = B.d; vb = B.vf;
        face_flux(uj, cj, C.ef, ub, cb, B.ef, p, FPr, FQr);
        carried = true;
        carP = FPr;
        carQ = FQr;
      } else {  // mirror ghost (cliffs.f:145-152)
        ub = -uj; cb = cj; db = dj; vb = vj;
        FPr = R(-2) * cj * uj;
        FQr = -FPr;
      }
      const R inv_fm = geo_m.inv_fm, inv_fp = geo_m.inv_fp, dtx = geo_m.dtx;
      const R Hj = (C.fl & F_LAND) ? p.ground : C.H;  // h^2/g
      R cc = R(0);
      if (p.gcrough != R(0)) {  // "almost Manning" friction (cliffs.f:204)
        const R r = frsqrt(Hj);  // sqrt((u^2+v^2)/H)/H = |u,v| / H^1.5
        cc = p.gcrough * uj * fsqrt0(uj * uj + vj * vj) * (r * r * r);
      }
      const R sphr = R(8) * cj * uj * geo_m.scl;  // (P-Q)(P+Q)*scl
      const bool water = (dj > p.ground) && (da > p.ground) && (db > p.ground);
      R sdiff = R(0);
      const bool sonP = water && (ua + ca < R(0)) && (ub + cb > R(0));
      const bool sonQ = water && (ua - ca < R(0)) && (ub - cb > R(0));
      if (sonP || sonQ) sdiff = R(2) * p.g * (csqrt(dj * db) - csqrt(dj * da));
      const R isum = dtx * p.idt;  // 1/(fm+fp)
      // P equation (cliffs.f:223-234)
      R QpP = FPr * inv_fp, QmP = FPl * inv_fm, QsP;
      const R ejP = uj + cj;  // e_j/4
      if (sonP)
        QsP = (ejP * ((ub - ua) + R(2) * (cb - ca)) - sdiff) * isum;
      else
        QsP = R(0.5) * (QpP + QmP);
      QsP = QsP + ejP * dtx * (QmP - QpP);
      const R dP = -p.dt * (QsP + cc - sphr);
      // Q equation (cliffs.f:236-247)
      R QpQ = FQr * inv_fp, QmQ = FQl * inv_fm, QsQ;
      const R ejQ = uj - cj;
      if (sonQ)
        QsQ = (ejQ * ((ub - ua) - R(2) * (cb - ca)) - sdiff) * isum;
      else
        QsQ = R(0.5) * (QpQ + QmQ);
      QsQ = QsQ + ejQ * dtx * (QmQ - QpQ);
      const R dQ = -p.dt * (QsQ + cc + sphr);
      // tangential velocity (cliffs.f:249-250)
      const R Qv = (vb - vj) * inv_fp - (vj - va) * inv_fm;
      C.vn = vj - uj * dtx * ((vb - va) - Qv * (uj * p.dt + geo_m.dfpm));
      const R dc = R(0.25) * (dP - dQ);
      C.cn = cj + dc;
      C.un = uj + R(0.5) * (dP + dQ);
      C.en = eta_step(cj, C.ef, dc, dj, p);
    } else if (m == 1 && (C.fl & F_EW)) {
      // left edge (cliffs.f:288-308)
      C.cn = C.c; C.un = C.uf; C.vn = C.vf; C.en = C.ef;
      if ((B.fl & F_EW) && (eL.eta + C.d > p.ground)) {
        R FP, FQ;
        face_flux(C.uf, C.c, C.ef, B.uf, B.c, B.ef, p, FP, FQ);
        const R sphr = R(8) * C.c * C.uf * scl1;
        const R dQ = -p.dt * (FQ * inv_dx1 + sphr);
        const R cbnd = csqrt(p.g * (C.d + eL.eta));
        const R dP = (eL.un - C.uf) + R(2) * p.g * (eL.eta - C.ef) / (cbnd + C.c);
        C.vn = (C.uf < R(0)) ? C.vf - p.dt * (B.vf - C.vf) * C.uf * inv_dx1 : eL.vt;
        const R dc = R(0.25) * (dP - dQ);
        C.cn = C.c + dc;
        C.un = C.uf + R(0.5) * (dP + dQ);
        C.en = eta_step(C.c, C.ef, dc, C.d, p);
      }
    } else if (m == n && (C.fl & F_EW)) {
      // right edge (cliffs.f:309-329)
      C.cn = C.c; C.un = C.uf; C.vn = C.vf; C.en = C.ef;
      if ((D.fl & F_EW) && (eR.eta + C.d > p.ground)) {
        R FP, FQ;
        face_flux(D.uf, D.c, D.ef, C.uf, C.c, C.ef, p, FP, FQ);
        const R sphr = R(8) * C.c * C.uf * scln;
        const R dP = -p.dt * (FP * inv_dxn1 - sphr);
        const R cbnd = csqrt(p.g * (C.d + eR.eta));
        const R dQ = (eR.un - C.uf) - R(2) * p.g * (eR.eta - C.ef) / (cbnd + C.c);
        C.vn = (C.uf > R(0)) ? C.vf - p.dt * (C.vf - D.vf) * C.uf * inv_dxn1 : eR.vt;
        const R dc = R(0.25) * (dP - dQ);
        C.cn = C.c + dc;
        C.un = C.uf + R(0.5) * (dP + dQ);
        C.en = eta_step(C.c, C.ef, dc, C.d, p);
      }
    }
    fpr_ok = carried;
    fpr_P = carP;
    fpr_Q = carQ;
    // ---- stage D: output cell o = k-3
    const int o = k - 3;
    if (!(D.fl & F_PRESENT)) return false;
    if (D.fl & F_EW) {
      R cO = D.cn, uO = D.un, eO = D.en;
      if (o >= 2 && o <= n - 1) {
        // shoreline angle limiter on newly wetted cells (cliffs.f:264-285)
        if ((D.fl & F_L) && !(E.fl & F_EW)) {
          const R hj = (o + 1 <= n - 1) ? C.cn : C.c;
          const R uj = (o + 1 <= n - 1) ? C.un : C.uf;
          if (p.sqr2 * cO > hj) {
            cO = hj / p.sqr2;
            eO = eta_from_c(cO, D.d, p);
          }
          if (uO < uj) uO = uj;
        } else if ((D.fl & F_R) && !(C.fl & F_EW)) {
          const R hj = (o - 1 >= 2) ? E.cn : E.c;
          const R uj = (o - 1 >= 2) ? E.un : E.uf;
          if (p.sqr2 * cO > hj) {
            cO = hj / p.sqr2;
            eO = eta_from_c(cO, D.d, p);
          }
          if (uO > uj) uO = uj;
        }
      }
      out.eta = eO;
      out.u = uO;
      out.v = D.vn;
    } else if (wet) {  // newland in a line with water: h=u=v=0 (cliffs.f:118-122)
      out.eta = -D.d;
      out.u = R(0);
      out.v = R(0);
    } else {  // fully dry line: untouched
      out.eta = D.eta;
      out.u = D.u;
      out.v = D.v;
    }
    (void)o;
    return true;
  }

  // push() for a stretch where cells k-3..k are all wet (H > ground) and
  // interior (2 <= k-3, k <= n-1): no flooding, no shoreline ghost, no
  // limiter, no edge.  Leaves the ring exactly as push() would.
  CL_HD OutCell<R> push_fast(R d, R eta, R u, R v, const Geo<R>& geo_m) {
    re = rd;
    rd = rc;
    rc = rb;
    rb = ra;
    RCell<R>& A = ra;
    RCell<R>& B = rb;
    RCell<R>& C = rc;
    RCell<R>& D = rd;
    A.d = d;
    A.eta = eta;
    A.u = u;
    A.v = v;
    A.H = d + eta;
    A.fl = F_PRESENT;
    B.c = fsqrt_pos(p.g * B.H);
    B.ef = B.eta;
    B.uf = B.u;
    B.vf = B.v;
    B.fl = F_PRESENT | F_EW;
    // interior VTCS-2 update of C with real neighbours D (left), B (right)
    R FPl, FQl, FPr, FQr;
    if (fpr_ok) {
      FPl = fpr_P;
      FQl = fpr_Q;
    } else {
      face_flux(D.uf, D.c, D.ef, C.uf, C.c, C.ef, p, FPl, FQl);
    }
    face_flux(C.uf, C.c, C.ef, B.uf, B.c, B.ef, p, FPr, FQr);
    fpr_ok = true;
    fpr_P = FPr;
    fpr_Q = FQr;
    const CellState<R> a{D.uf, D.c, D.ef, D.d, D.vf, D.H};
    const CellState<R> j{C.uf, C.c, C.ef, C.d, C.vf, C.H};
    const CellState<R> b{B.uf, B.c, B.ef, B.d, B.vf, B.H};
    const OutCell<R> r = interior_update(a, j, b, FPl, FQl, FPr, FQr, geo_m, p, &C.cn);
    C.en = r.eta;
    C.un = r.u;
    C.vn = r.v;
    return OutCell<R>{D.en, D.un, D.vn};
  }
};

}  // namespace cliffs
