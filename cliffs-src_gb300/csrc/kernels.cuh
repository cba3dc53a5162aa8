// kernels.cuh -- device kernels of the Cliffs GB300 library.
//
// Layout in HBM (one grid): every field is an FP32 array of ny rows with a
// row pitch of `pitch` floats (nx rounded up to 32, 128-byte aligned rows), x
// fastest like the Fortran module arrays.  State is (eta, xvel, yvel) in two
// ping-pong copies; dep is read-only; hmax is kept as the maximum eta and
// velmax as the maximum u^2+v^2.
//
// Line wetness bitmaps: a sweep leaves every line of the NEXT sweep "untouched"
// when that line holds no wet cell (cliffs.f:113).  Each sweep therefore
// writes a bitmap of wet cells of its output in the layout of the next
// sweep's lines: word (line, block) has bit b set when cell 32*block+b of that
// line is wet.  rows layout: word index (j-1)*ceil(nx/32) + (i-1)/32;
// cols layout: word index (i-1)*ceil(ny/32) + (j-1)/32.
#pragma once
#include <cstdint>

#include "march.cuh"

namespace cliffs {

struct SweepParams {
  int pitch;
  int n;       // line length (nx for the x-sweep, ny for the y-sweep)
  int nlines;  // number of lines (ny for x, nx for y)
  int lo, hi;  // swept lines, 1-based; other lines are copied through
  int seg;     // output cells per warp work item, multiple of 32
  const float* dep;
  const float* eta_in;
  const float* xu_in;
  const float* yv_in;
  float* eta_out;
  float* xu_out;
  float* yv_out;
  float* hmax;    // max eta, nullptr when the max-wave update is not fused
  float* velmax;  // max u^2+v^2
  const uint32_t* bm_in;
  int ld_in;
  uint32_t* bm_out;
  int ld_out;
  int bm_mode;  // 0: ballot across lines (next sweep is the other direction)
                // 1: accumulate along the line (next sweep is the same)
  const float4* geo;  // per position m: 1/dx(m-1), 1/dx(m), dt/(dx(m-1)+dx(m)), dx(m)-dx(m-1)
  const float* scl;   // per position metric term (y-sweep), nullptr = 0
  const float2* lscale;  // per line (alpha, 1/alpha) (x-sweep), nullptr = 1
  float inv_dx1, inv_dxn1;
  // boundary forcing: records A (low edge) and B (high edge), (len,3,nt) FP64
  const double* feedA;
  const double* feedB;
  int feed_len;
  int irec;   // 1-based, tinput(irec-1) <= t < tinput(irec)
  double cc;  // lerp weight of record irec-1
  Phys<float> ph;
  unsigned* status;
};

template <int DIR>
__device__ __forceinline__ size_t cell_index(int L, int k, int pitch) {
  // DIR 0: line L is row j, position k is column i; DIR 1: line L is column i
  return DIR == 0 ? (size_t)(L - 1) * (size_t)pitch + (size_t)(k - 1)
                  : (size_t)(k - 1) * (size_t)pitch + (size_t)(L - 1);
}

// One warp per work item: 32 consecutive lines x one segment of `seg` output
// cells.  Each lane marches its own line through the segment with a 3-cell
// halo on both sides (cliffs.f:17-346 via LineMarch).
template <int DIR>
__global__ void __launch_bounds__(128) sweep_kernel(const SweepParams P) {
  const int lane = threadIdx.x & 31;
  const int gw = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int nlb = (P.nlines + 31) >> 5;
  const int nseg = (P.n + P.seg - 1) / P.seg;
  if (gw >= nlb * nseg) return;  // warp-uniform
  const int lb = gw / nseg;
  const int sg = gw - lb * nseg;
  const int L = (lb << 5) + lane + 1;
  const int n = P.n;
  const bool active = L <= P.nlines;
  const bool swept = active && L >= P.lo && L <= P.hi;
  const int o0 = sg * P.seg + 1;
  const int o1 = min(o0 + P.seg - 1, n);

  // A line with no wet cell is left untouched (cliffs.f:113).
  bool wet = false;
  if (swept) {
    const uint32_t* w = P.bm_in + (size_t)(L - 1) * (size_t)P.ld_in;
    const int blo = (max(1, o0 - 1) - 1) >> 5;
    const int bhi = (min(n, o1 + 1) - 1) >> 5;
    uint32_t acc = 0;
    for (int b = blo; b <= bhi; ++b) acc |= w[b];
    if (!acc) {
      const int nb = (n + 31) >> 5;
      for (int b = 0; b < nb && !acc; ++b) acc |= w[b];
    }
    wet = acc != 0u;
  }

  LineMarch<float> M;
  M.init(P.ph, n, wet);
  float alpha = 1.f, ialpha = 1.f;
  if (DIR == 0 && P.lscale != nullptr && active) {
    const float2 s = P.lscale[L - 1];
    alpha = s.x;
    ialpha = s.y;
  }
  M.inv_dx1 = P.inv_dx1 * ialpha;
  M.inv_dxn1 = P.inv_dxn1 * ialpha;
  M.scl1 = P.scl ? P.scl[0] : 0.f;
  M.scln = P.scl ? P.scl[n - 1] : 0.f;
  M.eL = EdgeVals<float>{0.f, 0.f, 0.f};
  M.eR = EdgeVals<float>{0.f, 0.f, 0.f};
  if (active && (o0 == 1 || o1 == n) && (P.feedA || P.feedB)) {
    // edge1/edge2 = lerp of the forcing records (cliffs_main.f:318-339)
    const int len = P.feed_len;
    const size_t r0 = (size_t)(P.irec - 2) * 3 * (size_t)len;
    const size_t r1 = (size_t)(P.irec - 1) * 3 * (size_t)len;
    const double cc = P.cc;
    const int cn = DIR == 0 ? 0 : 1;  // normal velocity component (iu)
    const int ct = DIR == 0 ? 1 : 0;  // tangential component (3-iu)
    auto val = [&](const double* A, int c) -> float {
      const size_t b = (size_t)(L - 1) + (size_t)c * (size_t)len;
      return (float)(A[b + r0] * cc + A[b + r1] * (1.0 - cc));
    };
    if (o0 == 1 && P.feedA) M.eL = EdgeVals<float>{val(P.feedA, cn), val(P.feedA, ct), val(P.feedA, 2)};
    if (o1 == n && P.feedB) M.eR = EdgeVals<float>{val(P.feedB, cn), val(P.feedB, ct), val(P.feedB, 2)};
  }

  const int kb = max(1, o0 - 3);
  const int ke = o1 + 3;
  uint32_t acc_bits = 0;
  bool bad = false;
#pragma unroll 2
  for (int k = kb; k <= ke; ++k) {
    float d = 0.f, e = 0.f, u = 0.f, v = 0.f;
    if (active && k <= n) {
      const size_t q = cell_index<DIR>(L, k, P.pitch);
      d = __ldg(P.dep + q);
      e = __ldg(P.eta_in + q);
      const float xu = __ldg(P.xu_in + q);
      const float yv = __ldg(P.yv_in + q);
      u = DIR == 0 ? xu : yv;
      v = DIR == 0 ? yv : xu;
    }
    Geo<float> g{0.f, 0.f, 0.f, 0.f, 0.f};
    const int m = k - 2;
    if (m >= 2 && m <= n - 1) {
      const float4 gg = __ldg(P.geo + (m - 1));
      g.inv_fm = gg.x * ialpha;
      g.inv_fp = gg.y * ialpha;
      g.dtx = gg.z * ialpha;
      g.dfpm = gg.w * alpha;
      g.scl = P.scl ? __ldg(P.scl + (m - 1)) : 0.f;
    }
    OutCell<float> oc;
    const bool has = M.push(k, d, e, u, v, g, oc);
    const int o = k - 3;
    if (has && o >= o0) {  // warp-uniform
      float eo, uo, vo;
      if (swept) {
        eo = oc.eta;
        uo = oc.u;
        vo = oc.v;
      } else {
        eo = M.rd.eta;
        uo = M.rd.u;
        vo = M.rd.v;
      }
      const float xo = DIR == 0 ? uo : vo;
      const float yo = DIR == 0 ? vo : uo;
      bool wetout = false;
      if (active) {
        const size_t q = cell_index<DIR>(L, o, P.pitch);
        P.eta_out[q] = eo;
        P.xu_out[q] = xo;
        P.yv_out[q] = yo;
        wetout = (M.rd.d + eo) > P.ph.ground;
        if (P.hmax) {  // max-wave update (cliffs_main.f:347-355)
          if (eo > P.hmax[q]) P.hmax[q] = eo;
          const float s = xo * xo + yo * yo;
          if (s > P.velmax[q]) P.velmax[q] = s;
        }
        bad |= !(isfinite(eo) && isfinite(xo) && isfinite(yo));
      }
      if (P.bm_mode == 0) {
        const unsigned b = __ballot_sync(0xffffffffu, wetout);
        if (lane == 0) P.bm_out[(size_t)(o - 1) * (size_t)P.ld_out + lb] = b;
      } else {
        acc_bits |= (wetout ? 1u : 0u) << ((o - 1) & 31);
        if ((o & 31) == 0 || o == o1) {
          if (active) P.bm_out[(size_t)(L - 1) * (size_t)P.ld_out + ((o - 1) >> 5)] = acc_bits;
          acc_bits = 0;
        }
      }
    }
  }
  if (bad) atomicOr(P.status, 1u);
}

}  // namespace cliffs
