// sweep.cuh -- the two kernels of one dimensional sweep (cliffs.f:17-346 over
// every line of the grid, cliffs_main.f:325-344).
//
// fast kernel: one thread per 4 consecutive cells of a line.  It loads the
//   6-cell window (the 4 cells and one neighbour on each side) into registers
//   (x-sweep: float4 loads along the row plus two shuffled halo cells;
//   y-sweep: 6 coalesced row loads of its column), and finishes every cell
//   whose own update needs no wet/dry logic:
//     - a cell with both neighbours wet (all three H > ground) gets the plain
//       VTCS-2 interior update (no flooding, no shoreline ghost, no limiter);
//     - a dry cell between dry neighbours that already holds the zero state
//       stays as it is (the reference zeroes it, or leaves the whole line
//       untouched: both give the same values).
//   Every other cell (shoreline, line ends, dried cells with residual state)
//   goes to a worklist.
// general kernel: one thread per worklist cell replays the full line update
//   (LineMarch: flooding, mirror ghosts, angle limiter, open/forced edges) over
//   the cell's window of +-3 neighbours and writes that one cell.
//
// The worklist is the only scratch memory: (line, position) pairs and a
// counter per sweep parity.  A fast kernel zeroes the counter of the other
// parity, which the previous sweep's general kernel has finished with.
#pragma once
#include <cstdint>

#include "march.cuh"

namespace cliffs {

struct SweepArgs {
  int pitch;
  int n;       // line length (nx for the x-sweep, ny for the y-sweep)
  int nlines;  // number of lines (ny for x, nx for y)
  int lo, hi;  // swept lines, 1-based; other lines are copied through
  const float* dep;
  const float* eta;
  const float* xu;
  const float* yv;
  float* eta_o;
  float* xu_o;
  float* yv_o;
  float* hmax;    // max eta, nullptr when the max-wave update is not fused
  float* velmax;  // max u^2+v^2
  const float4* geo;  // per position m: 1/dx(m-1), 1/dx(m), dt/(dx(m-1)+dx(m)), dx(m)-dx(m-1)
  int geo_uniform;    // every interior position has geo0
  float4 geo0;
  const float* scl;      // per position metric term (y-sweep), nullptr = 0
  const float2* lscale;  // per line (alpha, 1/alpha) (x-sweep), nullptr = 1
  float inv_dx1, inv_dxn1;
  // boundary forcing: records A (low edge) and B (high edge), (len,3,nt) FP64
  const double* feedA;
  const double* feedB;
  int feed_len;
  int irec;
  double cc;
  Phys<float> ph;
  uint32_t* list;       // worklist: (line-1)*n + (position-1)
  uint32_t* count;      // worklist length of this sweep
  uint32_t* count_next; // the other parity's counter, zeroed by the fast kernel
  unsigned* status;
};

enum : unsigned { ST_NAN = 1u };

template <int DIR>
__device__ __forceinline__ size_t cidx(int L, int k, int pitch) {
  // DIR 0: line L is row j, position k is column i; DIR 1: line L is column i
  return DIR == 0 ? (size_t)(L - 1) * (size_t)pitch + (size_t)(k - 1)
                  : (size_t)(k - 1) * (size_t)pitch + (size_t)(L - 1);
}

__device__ __forceinline__ Geo<float> geo_at(const SweepArgs& A, int m, float alpha, float ialpha) {
  float4 g = A.geo_uniform ? A.geo0 : __ldg(A.geo + (m - 1));
  Geo<float> r;
  r.inv_fm = g.x * ialpha;
  r.inv_fp = g.y * ialpha;
  r.dtx = g.z * ialpha;
  r.dfpm = g.w * alpha;
  r.scl = A.scl ? __ldg(A.scl + (m - 1)) : 0.f;
  return r;
}

template <int DIR>
__device__ __forceinline__ void store_out(const SweepArgs& A, size_t q, float eo, float uo, float vo,
                                          bool& bad) {
  const float xo = DIR == 0 ? uo : vo;
  const float yo = DIR == 0 ? vo : uo;
  A.eta_o[q] = eo;
  A.xu_o[q] = xo;
  A.yv_o[q] = yo;
  if (A.hmax) {  // max-wave update (cliffs_main.f:347-355)
    if (eo > A.hmax[q]) A.hmax[q] = eo;
    const float s2 = xo * xo + yo * yo;
    if (s2 > A.velmax[q]) A.velmax[q] = s2;
  }
  bad |= !isfinite(eo + xo + yo);
}

// Warp-aggregated append to the worklist.
__device__ __forceinline__ void enqueue(const SweepArgs& A, bool want, uint32_t entry) {
  const unsigned m = __ballot_sync(0xffffffffu, want);
  if (!m) return;
  const int lane = threadIdx.x & 31;
  const int leader = __ffs(m) - 1;
  uint32_t base = 0;
  if (lane == leader) base = atomicAdd(A.count, (uint32_t)__popc(m));
  base = __shfl_sync(0xffffffffu, base, leader);
  if (want) A.list[base + __popc(m & ((1u << lane) - 1u))] = entry;
}

constexpr int kCellsPerThread = 4;

template <int DIR>
__global__ void __launch_bounds__(256) fast_kernel(const SweepArgs A) {
  if (blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0) *A.count_next = 0u;
  const int lane = threadIdx.x & 31;
  const int n = A.n;
  int L, i0;  // line, first position (1-based)
  if (DIR == 0) {
    L = blockIdx.y + 1;
    i0 = (blockIdx.x * blockDim.x + threadIdx.x) * kCellsPerThread + 1;
  } else {
    L = blockIdx.y * 32 + lane + 1;
    i0 = (blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) * kCellsPerThread + 1;
  }
  const bool active = L <= A.nlines && i0 <= n;  // x-sweep: warp-uniform in L
  const bool swept = active && L >= A.lo && L <= A.hi;
  // window w[0..5] = positions i0-1 .. i0+4
  float d[6], e[6], u[6], v[6];
  if (DIR == 0) {
    // float4 along the row: positions i0..i0+3; halo cells from the neighbours
    const size_t q0 = cidx<0>(min(L, A.nlines), i0, A.pitch);
    float4 D4 = make_float4(0, 0, 0, 0), E4 = D4, X4 = D4, Y4 = D4;
    if (active) {
      D4 = __ldg(reinterpret_cast<const float4*>(A.dep + q0));
      E4 = __ldg(reinterpret_cast<const float4*>(A.eta + q0));
      X4 = __ldg(reinterpret_cast<const float4*>(A.xu + q0));
      Y4 = __ldg(reinterpret_cast<const float4*>(A.yv + q0));
    }
    d[1] = D4.x; d[2] = D4.y; d[3] = D4.z; d[4] = D4.w;
    e[1] = E4.x; e[2] = E4.y; e[3] = E4.z; e[4] = E4.w;
    u[1] = X4.x; u[2] = X4.y; u[3] = X4.z; u[4] = X4.w;
    v[1] = Y4.x; v[2] = Y4.y; v[3] = Y4.z; v[4] = Y4.w;
    d[0] = __shfl_up_sync(0xffffffffu, D4.w, 1);
    e[0] = __shfl_up_sync(0xffffffffu, E4.w, 1);
    u[0] = __shfl_up_sync(0xffffffffu, X4.w, 1);
    v[0] = __shfl_up_sync(0xffffffffu, Y4.w, 1);
    d[5] = __shfl_down_sync(0xffffffffu, D4.x, 1);
    e[5] = __shfl_down_sync(0xffffffffu, E4.x, 1);
    u[5] = __shfl_down_sync(0xffffffffu, X4.x, 1);
    v[5] = __shfl_down_sync(0xffffffffu, Y4.x, 1);
    if (active && lane == 0 && i0 > 1) {
      d[0] = __ldg(A.dep + q0 - 1);
      e[0] = __ldg(A.eta + q0 - 1);
      u[0] = __ldg(A.xu + q0 - 1);
      v[0] = __ldg(A.yv + q0 - 1);
    }
    if (active && lane == 31 && i0 + 4 <= n) {
      d[5] = __ldg(A.dep + q0 + 4);
      e[5] = __ldg(A.eta + q0 + 4);
      u[5] = __ldg(A.xu + q0 + 4);
      v[5] = __ldg(A.yv + q0 + 4);
    }
  } else {
#pragma unroll
    for (int w = 0; w < 6; ++w) {
      const int k = i0 - 1 + w;
      d[w] = e[w] = u[w] = v[w] = 0.f;
      if (active && k >= 1 && k <= n) {
        const size_t q = cidx<1>(L, k, A.pitch);
        d[w] = __ldg(A.dep + q);
        e[w] = __ldg(A.eta + q);
        v[w] = __ldg(A.xu + q);  // tangential in the y-sweep
        u[w] = __ldg(A.yv + q);  // normal
      }
    }
  }
  bool bad = false;
  unsigned need = 0u;  // bit r: cell i0+r goes to the general kernel
  if (active && !swept) {  // lines not swept are copied through
#pragma unroll
    for (int r = 0; r < kCellsPerThread; ++r) {
      const int k = i0 + r;
      if (k <= n) store_out<DIR>(A, cidx<DIR>(L, k, A.pitch), e[r + 1], u[r + 1], v[r + 1], bad);
    }
  } else if (active) {
    const Phys<float>& p = A.ph;
    float alpha = 1.f, ialpha = 1.f;
    if (DIR == 0 && A.lscale != nullptr) {
      const float2 s = A.lscale[L - 1];
      alpha = s.x;
      ialpha = s.y;
    }
    bool wet[6];
    float H[6], c[6];
#pragma unroll
    for (int w = 0; w < 6; ++w) {
      const int k = i0 - 1 + w;
      H[w] = d[w] + e[w];
      wet[w] = (k >= 1 && k <= n) && H[w] > p.ground;
      c[w] = fsqrt_pos(p.g * fmaxf(H[w], p.ground));
    }
    float FP[5], FQ[5];  // face fluxes between window cells w and w+1
#pragma unroll
    for (int f = 0; f < 5; ++f) face_flux(u[f], c[f], e[f], u[f + 1], c[f + 1], e[f + 1], p, FP[f], FQ[f]);
#pragma unroll
    for (int r = 0; r < kCellsPerThread; ++r) {
      const int k = i0 + r;
      const int w = r + 1;
      if (k <= n) {
        const size_t q = cidx<DIR>(L, k, A.pitch);
        if (k >= 2 && k <= n - 1 && wet[w - 1] && wet[w] && wet[w + 1]) {
          const CellState<float> a{u[w - 1], c[w - 1], e[w - 1], d[w - 1], v[w - 1], H[w - 1]};
          const CellState<float> j{u[w], c[w], e[w], d[w], v[w], H[w]};
          const CellState<float> b{u[w + 1], c[w + 1], e[w + 1], d[w + 1], v[w + 1], H[w + 1]};
          float cn;
          const OutCell<float> o =
              interior_update(a, j, b, FP[w - 1], FQ[w - 1], FP[w], FQ[w], geo_at(A, k, alpha, ialpha), p, &cn);
          store_out<DIR>(A, q, o.eta, o.u, o.v, bad);
        } else if (!wet[w] && !wet[w - 1] && !wet[w + 1] && H[w] == 0.f && u[w] == 0.f && v[w] == 0.f) {
          store_out<DIR>(A, q, e[w], u[w], v[w], bad);  // dry, zero state: unchanged either way
        } else {
          need |= 1u << r;
        }
      }
    }
  }
#pragma unroll
  for (int r = 0; r < kCellsPerThread; ++r)
    enqueue(A, (need >> r) & 1u, (uint32_t)(L - 1) * (uint32_t)n + (uint32_t)(i0 + r - 1));
  if (bad) atomicOr(A.status, ST_NAN);
}

// One thread per worklist cell: the full line update over its +-3 window.
template <int DIR>
__global__ void __launch_bounds__(128) general_kernel(const SweepArgs A) {
  const uint32_t cnt = *A.count;
  const int n = A.n;
  for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < cnt; t += gridDim.x * blockDim.x) {
    const uint32_t ent = A.list[t];
    const int L = (int)(ent / (uint32_t)n) + 1;
    const int o = (int)(ent % (uint32_t)n) + 1;
    const Phys<float>& p = A.ph;
    // Does the line hold a wet cell (cliffs.f:113)?  The +-3 window usually
    // answers; a cell whose window is all dry needs the answer only when it
    // holds a non-zero residual state, and then the whole line is scanned.
    bool wet = false, need = false;
    for (int k = max(1, o - 3); k <= min(n, o + 3); ++k) {
      const size_t q = cidx<DIR>(L, k, A.pitch);
      wet |= __ldg(A.dep + q) + __ldg(A.eta + q) > p.ground;
    }
    if (!wet) {
      const size_t q = cidx<DIR>(L, o, A.pitch);
      need = (__ldg(A.dep + q) + __ldg(A.eta + q)) != 0.f || __ldg(A.xu + q) != 0.f || __ldg(A.yv + q) != 0.f;
      for (int k = 1; need && !wet && k <= n; ++k) {
        const size_t q2 = cidx<DIR>(L, k, A.pitch);
        wet |= __ldg(A.dep + q2) + __ldg(A.eta + q2) > p.ground;
      }
    }
    float alpha = 1.f, ialpha = 1.f;
    if (DIR == 0 && A.lscale != nullptr) {
      const float2 s = A.lscale[L - 1];
      alpha = s.x;
      ialpha = s.y;
    }
    LineMarch<float> M;
    M.init(p, n, wet);
    M.inv_dx1 = A.inv_dx1 * ialpha;
    M.inv_dxn1 = A.inv_dxn1 * ialpha;
    M.scl1 = A.scl ? A.scl[0] : 0.f;
    M.scln = A.scl ? A.scl[n - 1] : 0.f;
    M.eL = EdgeVals<float>{0.f, 0.f, 0.f};
    M.eR = EdgeVals<float>{0.f, 0.f, 0.f};
    if ((o <= 4 || o >= n - 3) && (A.feedA || A.feedB)) {
      // edge1/edge2 = lerp of the forcing records (cliffs_main.f:318-339)
      const int len = A.feed_len;
      const size_t r0 = (size_t)(A.irec - 2) * 3 * (size_t)len;
      const size_t r1 = (size_t)(A.irec - 1) * 3 * (size_t)len;
      const double cc = A.cc;
      const int cn = DIR == 0 ? 0 : 1;  // normal velocity component (iu)
      const int ct = DIR == 0 ? 1 : 0;  // tangential component (3-iu)
      auto val = [&](const double* F, int comp) -> float {
        const size_t b = (size_t)(L - 1) + (size_t)comp * (size_t)len;
        return (float)(F[b + r0] * cc + F[b + r1] * (1.0 - cc));
      };
      if (A.feedA) M.eL = EdgeVals<float>{val(A.feedA, cn), val(A.feedA, ct), val(A.feedA, 2)};
      if (A.feedB) M.eR = EdgeVals<float>{val(A.feedB, cn), val(A.feedB, ct), val(A.feedB, 2)};
    }
    OutCell<float> res{0.f, 0.f, 0.f};
    for (int k = max(1, o - 3); k <= o + 3; ++k) {
      float dd = 0.f, ee = 0.f, uu = 0.f, vv = 0.f;
      if (k <= n) {
        const size_t q = cidx<DIR>(L, k, A.pitch);
        dd = __ldg(A.dep + q);
        ee = __ldg(A.eta + q);
        const float xu = __ldg(A.xu + q), yv = __ldg(A.yv + q);
        uu = DIR == 0 ? xu : yv;
        vv = DIR == 0 ? yv : xu;
      }
      const int m = k - 2;
      Geo<float> g{0.f, 0.f, 0.f, 0.f, 0.f};
      if (m >= 2 && m <= n - 1) g = geo_at(A, m, alpha, ialpha);
      OutCell<float> oc;
      if (M.push(k, dd, ee, uu, vv, g, oc) && k - 3 == o) res = oc;
    }
    bool bad = false;
    store_out<DIR>(A, cidx<DIR>(L, o, A.pitch), res.eta, res.u, res.v, bad);
    if (bad) atomicOr(A.status, ST_NAN);
  }
}

}  // namespace cliffs
