// march.cuh -- the VTCS-2 update of one line cell, in the forms the sweep
// kernels use.
//
// Restates cliffs.f:17-346 (subroutine cliffs) cell by cell:
//   interior_update     VTCS-2 interior update (cliffs.f:175-262)
//   edge_left/right     open or forced line ends (cliffs.f:287-329)
//   general_cell        the whole of cliffs.f:56-329 for one cell: flooding
//                       (cliffs.f:74-111), newland (118-122), mirror ghosts
//                       (137-152), the update, the shoreline angle limiter
//                       (264-285)
//
// The serial segment scan of the reference is replaced by per-cell rules that
// depend on cells i-1..i+1 only; the oracle's orc_line_local proves them
// bit-identical to the scan in FP64.  Segments are the maximal runs of
// wet-or-flooded cells; an interior cell whose neighbour is not in its run uses
// the mirror ghost of itself (cliffs.f:137-152).  A line without any wet cell
// is left untouched (cliffs.f:113); the caller supplies that line flag.
//
// Stored state.  The reference carries celerity c = sqrt(gH) in FP64.  Here
// the surface is carried as one FP32 number per cell, the surface state s:
//   s = eta           where the bed is below datum (d >= 0, the sea),
//   s = H = d + eta   where it is above (d < 0, land).
// At sea eta keeps ~1e-7 m resolution whatever the depth, where c or H would
// lose it to the depth.  On land eta = H + |d| would keep only ulp(|d|) of a
// run-up film a few millimetres thick, and the rounding of every step's
// increment to that ulp is what drives an FP32 run-down away from FP64; H keeps
// full relative precision in the film.  Both forms move by the same increment
// (eta and H differ by the constant d), so the update is written once.
//
// The hydrostatic balance (1/8)(e2+ej)(p2-pj) - g(d2-dj) is rewritten with
// c^2 = g(d+eta) as
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

// Single operations, each rounded once, as written: on the GPU they are
// intrinsics, which the compiler neither fuses nor splits, so every kernel
// that inlines the interior update (flat or general geometry, single grid or
// batched) rounds it the same way.
CL_HD float add_rn(float x, float y) {
#ifdef __CUDA_ARCH__
  return __fadd_rn(x, y);
#else
  return x + y;
#endif
}
CL_HD float sub_rn(float x, float y) {
#ifdef __CUDA_ARCH__
  return __fsub_rn(x, y);
#else
  return x - y;
#endif
}
CL_HD float mul_rn(float x, float y) {
#ifdef __CUDA_ARCH__
  return __fmul_rn(x, y);
#else
  return x * y;
#endif
}
CL_HD float fma_rn(float a, float b, float c) {  // a * b + c
#ifdef __CUDA_ARCH__
  return __fmaf_rn(a, b, c);
#else
  return std::fma(a, b, c);
#endif
}
CL_HD double add_rn(double x, double y) { return x + y; }
CL_HD double sub_rn(double x, double y) { return x - y; }
CL_HD double mul_rn(double x, double y) { return x * y; }
CL_HD double fma_rn(double a, double b, double c) {
#ifdef __CUDA_ARCH__
  return __fma_rn(a, b, c);
#else
  return std::fma(a, b, c);
#endif
}

// x / y where ~2 ulp is enough (y away from 0 and from huge values)
CL_HD float fdiv(float x, float y) {
#ifdef __CUDA_ARCH__
  return __fdividef(x, y);
#else
  return x / y;
#endif
}
CL_HD double fdiv(double x, double y) { return x / y; }

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

// Surface state s <-> (eta, H) for bed elevation -d (see the file header).
template <typename R>
CL_HD R eta_of(R s, R d) {
  return d < R(0) ? s - d : s;
}
template <typename R>
CL_HD R depth_of(R s, R d) {
  return d < R(0) ? s : d + s;
}
template <typename R>
CL_HD R state_from_depth(R H, R d) {
  return d < R(0) ? H : H - d;
}

template <typename R>
struct EdgeVals {
  R un, vt, eta;  // feed normal velocity, tangential velocity, elevation
};

template <typename R>
struct OutCell {
  R s, u, v;  // final surface state, normal and tangential velocity
};

template <typename R>
CL_HD void face_flux(R ul, R cl, R el, R ur, R cr, R er, const Phys<R>& p,
                     R& FP, R& FQ) {
  // (1/8)(e_l+e_r)(P_r-P_l) - g(d_r-d_l), e = 3P+Q = 4(u+c), and the Q analogue
  const R U = add_rn(ul, ur), C = add_rn(cl, cr), du = sub_rn(ur, ul), dc = sub_rn(cr, cl);
  const R gde = mul_rn(p.g, sub_rn(er, el));
  const R Udc = mul_rn(U, dc);
  FP = fma_rn(mul_rn(R(0.5), add_rn(U, C)), du, add_rn(gde, Udc));
  FQ = fma_rn(mul_rn(R(0.5), sub_rn(U, C)), du, sub_rn(gde, Udc));
}

// Surface state of celerity c (sign kept: H = c|c|/g).
template <typename R>
CL_HD R state_from_c(R c, R d, const Phys<R>& p) {
  return state_from_depth(mul_rn(mul_rn(c, c < R(0) ? -c : c), p.ginv), d);
}

// State of one cell as the interior update sees it (after flooding).  e and H
// are both given; the one the cell stores (eta at sea, H on land) is exact.
template <typename R>
struct CellState {
  R u, c, e, d, v, H;  // normal velocity, celerity, eta, depth, tangential, H
};

// New surface state after the celerity c0 of cell j moved by dc: the exact
// increment dH = dc(2c0+dc)/g added to the stored form when both celerities
// are positive.
template <typename R>
CL_HD R state_step(const CellState<R>& j, R dc, const Phys<R>& p) {
  const R c0 = j.c, c1 = add_rn(c0, dc);
  if (c0 > R(0) && c1 > R(0)) return fma_rn(mul_rn(dc, fma_rn(R(2), c0, dc)), p.ginv, j.d < R(0) ? j.H : j.e);
  return state_from_c(c1, j.d, p);
}

struct NoFlux {};

// VTCS-2 interior update of cell j between real neighbours a (left) and b
// (right), cliffs.f:200-262, in the eta form.  FPl/FQl, FPr/FQr are the face
// fluxes (a,j) and (j,b).  Returns the new (s, u, v); *cn gets the new
// celerity.  TC = false leaves out the transcritical-point test, for callers
// that know no neighbour is supercritical (|u| <= c), where it cannot fire.
// SPH = false leaves out the metric term, for lines without one (geo.scl 0:
// the term is then a zero, and leaving it out can change at most the sign
// of a zero result).
template <typename R, bool TC = true, bool SPH = true>
CL_HD OutCell<R> interior_update(const CellState<R>& a, const CellState<R>& j, const CellState<R>& b,
                                 R FPl, R FQl, R FPr, R FQr, const Geo<R>& geo, const Phys<R>& p,
                                 R* cn_out) {
  const R uj = j.u, cj = j.c, vj = j.v, dj = j.d;
  const R inv_fm = geo.inv_fm, inv_fp = geo.inv_fp, dtx = geo.dtx;
  const R r = frsqrt(j.H);  // sqrt((u^2+v^2)/H)/H = |u,v| / H^1.5 (cliffs.f:204)
  const R cc = mul_rn(mul_rn(mul_rn(p.gcrough, uj), fsqrt0(fma_rn(uj, uj, mul_rn(vj, vj)))),
                      mul_rn(mul_rn(r, r), r));
  const R sphr = SPH ? mul_rn(mul_rn(mul_rn(R(8), cj), uj), geo.scl) : R(0);  // (P-Q)(P+Q)*scl
  const R ejP = add_rn(uj, cj), ejQ = sub_rn(uj, cj);
  const R QpP = mul_rn(FPr, inv_fp), QmP = mul_rn(FPl, inv_fm);
  const R QpQ = mul_rn(FQr, inv_fp), QmQ = mul_rn(FQl, inv_fm);
  R QsP = mul_rn(R(0.5), add_rn(QpP, QmP));
  R QsQ = mul_rn(R(0.5), add_rn(QpQ, QmQ));
  const bool sonP = TC && (a.u + a.c < R(0)) && (b.u + b.c > R(0));
  const bool sonQ = TC && (a.u - a.c < R(0)) && (b.u - b.c > R(0));
  if ((sonP || sonQ) && (dj > p.ground) && (a.d > p.ground) && (b.d > p.ground)) {
    // transcritical point (cliffs.f:228-232, 241-245)
    const R isum = mul_rn(dtx, p.idt);
    const R sdiff = mul_rn(mul_rn(R(2), p.g), sub_rn(fsqrt_pos(mul_rn(dj, b.d)), fsqrt_pos(mul_rn(dj, a.d))));
    const R du = sub_rn(b.u, a.u), dcl = sub_rn(b.c, a.c);
    if (sonP) QsP = mul_rn(sub_rn(mul_rn(ejP, fma_rn(R(2), dcl, du)), sdiff), isum);
    if (sonQ) QsQ = mul_rn(sub_rn(mul_rn(ejQ, fma_rn(R(-2), dcl, du)), sdiff), isum);
  }
  QsP = fma_rn(mul_rn(ejP, dtx), sub_rn(QmP, QpP), QsP);
  QsQ = fma_rn(mul_rn(ejQ, dtx), sub_rn(QmQ, QpQ), QsQ);
  // -dt (Qs + cc -/+ sphr); without the metric term the zero is left out
  const R qcP = add_rn(QsP, cc), qcQ = add_rn(QsQ, cc);
  const R mdt = -p.dt;
  const R dP = mul_rn(mdt, SPH ? sub_rn(qcP, sphr) : qcP);
  const R dQ = mul_rn(mdt, SPH ? add_rn(qcQ, sphr) : qcQ);
  const R Qv = fma_rn(sub_rn(b.v, vj), inv_fp, -mul_rn(sub_rn(vj, a.v), inv_fm));
  OutCell<R> o;
  const R vx = fma_rn(-Qv, fma_rn(uj, p.dt, geo.dfpm), sub_rn(b.v, a.v));
  o.v = fma_rn(-mul_rn(uj, dtx), vx, vj);
  const R dc = mul_rn(R(0.25), sub_rn(dP, dQ));
  *cn_out = add_rn(cj, dc);
  o.u = fma_rn(R(0.5), add_rn(dP, dQ), uj);
  o.s = state_step(j, dc, p);
  return o;
}

// Open / forced edge update of line cell 1 (cliffs.f:288-308): C is cell 1
// and B cell 2 (flood-modified), both wet or flooded.
template <typename R>
CL_HD void edge_left(const CellState<R>& C, const CellState<R>& B, const EdgeVals<R>& e, R inv_dx1, R scl1,
                     const Phys<R>& p, R& cn, R& un, R& vn, R& sn) {
  R FP, FQ;
  face_flux(C.u, C.c, C.e, B.u, B.c, B.e, p, FP, FQ);
  const R sphr = mul_rn(mul_rn(mul_rn(R(8), C.c), C.u), scl1);
  const R dQ = mul_rn(-p.dt, fma_rn(FQ, inv_dx1, sphr));
  const R cbnd = fsqrt_pos(mul_rn(p.g, add_rn(C.d, e.eta)));  // C.d + e.eta > ground: the caller's edge condition
  const R dP = add_rn(sub_rn(e.un, C.u), fdiv(mul_rn(mul_rn(R(2), p.g), sub_rn(e.eta, C.e)), add_rn(cbnd, C.c)));
  vn = (C.u < R(0)) ? sub_rn(C.v, mul_rn(mul_rn(mul_rn(p.dt, sub_rn(B.v, C.v)), C.u), inv_dx1)) : e.vt;
  const R dc = mul_rn(R(0.25), sub_rn(dP, dQ));
  cn = add_rn(C.c, dc);
  un = fma_rn(R(0.5), add_rn(dP, dQ), C.u);
  sn = state_step(C, dc, p);
}

// Open / forced edge update of line cell n (cliffs.f:309-329): D is cell n-1,
// C cell n.
template <typename R>
CL_HD void edge_right(const CellState<R>& D, const CellState<R>& C, const EdgeVals<R>& e, R inv_dxn1, R scln,
                      const Phys<R>& p, R& cn, R& un, R& vn, R& sn) {
  R FP, FQ;
  face_flux(D.u, D.c, D.e, C.u, C.c, C.e, p, FP, FQ);
  const R sphr = mul_rn(mul_rn(mul_rn(R(8), C.c), C.u), scln);
  const R dP = mul_rn(-p.dt, fma_rn(FP, inv_dxn1, -sphr));
  const R cbnd = fsqrt_pos(mul_rn(p.g, add_rn(C.d, e.eta)));  // C.d + e.eta > ground: the caller's edge condition
  const R dQ = sub_rn(sub_rn(e.un, C.u), fdiv(mul_rn(mul_rn(R(2), p.g), sub_rn(e.eta, C.e)), add_rn(cbnd, C.c)));
  vn = (C.u > R(0)) ? sub_rn(C.v, mul_rn(mul_rn(mul_rn(p.dt, sub_rn(C.v, D.v)), C.u), inv_dxn1)) : e.vt;
  const R dc = mul_rn(R(0.25), sub_rn(dP, dQ));
  cn = add_rn(C.c, dc);
  un = fma_rn(R(0.5), add_rn(dP, dQ), C.u);
  sn = state_step(C, dc, p);
}

// Raw input of one line cell; present iff 1 <= position <= n.
template <typename R>
struct RawCell {
  R d, s, u, v;  // depth, surface state, normal and tangential velocity
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
  R H[7], E[7];
#pragma unroll
  for (int t = 0; t < 7; ++t) {
    H[t] = depth_of(w[t].s, w[t].d);
    E[t] = eta_of(w[t].s, w[t].d);
    land[t] = !w[t].present || H[t] <= p.ground;
    Rf[t] = Lf[t] = false;
  }
#pragma unroll
  for (int t = 1; t <= 5; ++t) {
    if (w[t].present && land[t]) {
      Rf[t] = w[t - 1].present && !land[t - 1] && w[t - 1].u >= R(0) && (E[t - 1] + w[t].d > p.ground);
      Lf[t] = !Rf[t] && w[t + 1].present && !land[t + 1] && w[t + 1].u <= R(0) &&
              (E[t + 1] + w[t].d > p.ground);
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
      fm[t] = CellState<R>{w[t].u, fsqrt_pos(p.g * (H[t] > p.ground ? H[t] : p.ground)), E[t], w[t].d, w[t].v,
                           H[t]};
    }
  }
  OutCell<R> out;
  if (!ew[3]) {
    if (L.wet) {  // newland in a line with water: h=u=v=0 (cliffs.f:118-122)
      out.s = state_from_depth(R(0), w[3].d);
      out.u = R(0);
      out.v = R(0);
    } else {  // a line without water is left untouched (cliffs.f:113)
      out.s = w[3].s;
      out.u = w[3].u;
      out.v = w[3].v;
    }
    return out;
  }
  const int n = L.n;
  if (o == 1 || o == n) {
    // flood-modified value unless the edge condition holds
    out.s = (Rf[3] || Lf[3]) ? state_from_depth(p.ground, w[3].d) : w[3].s;
    out.u = fm[3].u;
    out.v = fm[3].v;
    R cn, un, vn, sn;
    if (o == 1 && n >= 2 && ew[4] && (L.eL.eta + w[3].d > p.ground)) {
      edge_left(fm[3], fm[4], L.eL, L.inv_dx1, L.scl1, p, cn, un, vn, sn);
      out.s = sn;
      out.u = un;
      out.v = vn;
    } else if (o == n && n >= 2 && ew[2] && (L.eR.eta + w[3].d > p.ground)) {
      edge_right(fm[2], fm[3], L.eR, L.inv_dxn1, L.scln, p, cn, un, vn, sn);
      out.s = sn;
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
      out.s = state_from_c(cO, w[3].d, p);
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
      out.s = state_from_c(cO, w[3].d, p);
    }
    if (out.u > uj) out.u = uj;
  }
  return out;
}

}  // namespace cliffs
