// sweep.cuh -- the two kernels of one dimensional sweep: subroutine cliffs
// (cliffs.f:17-346) over every line of the grid (cliffs_main.f:325-344).
//
// fast kernel: one thread owns 4 consecutive cells of a line and loads the
//   6-cell window (the 4 cells and one neighbour on each side) into registers:
//   the x-sweep (lines are rows) with float4 loads along the row plus two
//   shuffled halo cells, the y-sweep (lines are columns) with 6 row loads that
//   are coalesced across the warp (lanes are neighbouring columns).  It
//   finishes every cell whose update needs no wet/dry logic:
//     - both neighbours wet (all three H > ground): the plain VTCS-2 interior
//       update (the open ocean, almost every cell);
//     - dry between dry neighbours and already at the zero state: unchanged
//       (the reference zeroes it, or leaves the whole line untouched: same
//       values);
//   and lists every other cell (shorelines, line ends, drying cells).
// general kernel: one thread per listed cell evaluates general_cell, the full
//   wet/dry rule set, on the raw cells o-3..o+3 and overwrites that cell.
//
// The worklist is the sweep's only scratch memory: (line, position) entries
// and one counter per sweep parity; the fast kernel zeroes the counter of the
// other parity, which the previous sweep's general kernel has finished with.
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
  const float* srf;  // surface state: eta where dep >= 0, water depth where dep < 0
  const float* xu;
  const float* yv;
  float* srf_o;
  float* xu_o;
  float* yv_o;
  float* hmax;    // max eta, nullptr when the max-wave update is not fused
  float* velmax;  // max u^2+v^2
  // x-sweep of a two-dimensional step: the max-wave fields updated with the
  // sweep's INPUT, the state the previous step ended with (nullptr: not)
  float* hmax_in;
  float* velmax_in;
  const float4* geo;  // per position m: 1/dx(m-1), 1/dx(m), dt/(dx(m-1)+dx(m)), dx(m)-dx(m-1)
  int geo_uniform;    // every interior position has geo0
  float4 geo0;
  const float* scl;      // per position metric term (y-sweep), nullptr = 0
  const float2* lscale;  // per line (alpha, 1/alpha) (x-sweep), nullptr = 1
  float inv_dx1, inv_dxn1;
  // forcing at the line ends for this step, 6 floats per line: normal
  // velocity, tangential velocity, eta at cell 1, then at cell n; nullptr =
  // still-water open edges
  const float* edges;
  Phys<float> ph;
  uint32_t* list;        // worklist: (line-1)*n + (position-1)
  uint32_t* count;       // worklist length of this sweep
  uint32_t* count_next;  // the other parity's counter, zeroed by the fast kernel
  // [0] status bits (ST_*); [1] the largest Courant number above 1 seen, as
  // float bits (0: none)
  unsigned* status;
};

enum : unsigned { ST_NAN = 1u, ST_CFL = 4u };

// Loads of the state fields (surface, u, v, max-wave).  A sweep kernel reads
// the fields another launch wrote, through the read-only path (COH = false).
// The batched persistent kernel (batch.cuh) reads fields that other blocks of
// the same launch wrote before a grid barrier: those loads go to L2
// (COH = true), where the writes are, not to a possibly stale L1 line.
template <bool COH>
__device__ __forceinline__ float ld_state(const float* p) {
  return COH ? __ldcg(p) : __ldg(p);
}
template <bool COH>
__device__ __forceinline__ float4 ld_state4(const float* p) {
  return COH ? __ldcg(reinterpret_cast<const float4*>(p)) : __ldg(reinterpret_cast<const float4*>(p));
}

template <int DIR>
__device__ __forceinline__ size_t cidx(int L, int k, int pitch) {
  // DIR 0: line L is row j, position k is column i; DIR 1: line L is column i
  return DIR == 0 ? (size_t)(L - 1) * (size_t)pitch + (size_t)(k - 1)
                  : (size_t)(k - 1) * (size_t)pitch + (size_t)(L - 1);
}

__device__ __forceinline__ Geo<float> geo_at(const SweepArgs& A, int m, float alpha, float ialpha) {
  Geo<float> r{0.f, 0.f, 0.f, 0.f, 0.f};
  if (m < 2 || m > A.n - 1) return r;
  const float4 g = A.geo_uniform ? A.geo0 : __ldg(A.geo + (m - 1));
  r.inv_fm = g.x * ialpha;
  r.inv_fp = g.y * ialpha;
  r.dtx = g.z * ialpha;
  r.dfpm = g.w * alpha;
  r.scl = A.scl ? __ldg(A.scl + (m - 1)) : 0.f;
  return r;
}

// Geometry of position m for the plain update: g0 is the line's uniform
// geometry, already scaled by the row factor; a non-uniform line reads its
// table.  Unlike geo_at there is no zeroing at the line ends: the plain update
// only keeps cells with 2 <= m <= n-1, and the caller clamps m to 1..n.
__device__ __forceinline__ Geo<float> geo_plain(const SweepArgs& A, int m, const Geo<float>& g0, float alpha,
                                                float ialpha) {
  Geo<float> r = g0;
  if (!A.geo_uniform) {
    const float4 g = __ldg(A.geo + (m - 1));
    r = Geo<float>{g.x * ialpha, g.y * ialpha, g.z * ialpha, g.w * alpha, 0.f};
  }
  r.scl = A.scl ? __ldg(A.scl + (m - 1)) : 0.f;
  return r;
}

// edge1 (cell 1, side 0) or edge2 (cell n, side 1) of line L.
__device__ __forceinline__ EdgeVals<float> edge_vals(const SweepArgs& A, int L, int side) {
  if (!A.edges) return EdgeVals<float>{0.f, 0.f, 0.f};
  const float* e = A.edges + (size_t)(L - 1) * 6 + side * 3;
  return EdgeVals<float>{e[0], e[1], e[2]};
}

// The cell's value through the full wet/dry rules (cliffs.f:56-329).
template <int DIR, bool COH>
__device__ __forceinline__ OutCell<float> general_path(const SweepArgs& A, int L, int o, float alpha, float ialpha,
                                                       const EdgeVals<float>& eL, const EdgeVals<float>& eR) {
  const int n = A.n;
  const Phys<float>& p = A.ph;
  RawCell<float> w[7];
  bool anywet = false;
#pragma unroll
  for (int t = 0; t < 7; ++t) {
    const int k = o - 3 + t;
    w[t] = RawCell<float>{0.f, 0.f, 0.f, 0.f, false};
    if (k >= 1 && k <= n) {
      const size_t q = cidx<DIR>(L, k, A.pitch);
      const float xu = ld_state<COH>(A.xu + q), yv = ld_state<COH>(A.yv + q);
      w[t] = RawCell<float>{__ldg(A.dep + q), ld_state<COH>(A.srf + q), DIR == 0 ? xu : yv, DIR == 0 ? yv : xu,
                            true};
      anywet |= depth_of(w[t].s, w[t].d) > p.ground;
    }
  }
  LineCtx<float> C;
  C.n = n;
  C.wet = anywet;
  if (!anywet && !(depth_of(w[3].s, w[3].d) == 0.f && w[3].u == 0.f && w[3].v == 0.f)) {
    // does the line hold a wet cell anywhere (cliffs.f:113)?
    for (int k = 1; k <= n && !C.wet; ++k) {
      const size_t q = cidx<DIR>(L, k, A.pitch);
      C.wet = depth_of(ld_state<COH>(A.srf + q), __ldg(A.dep + q)) > p.ground;
    }
  }
  C.eL = eL;
  C.eR = eR;
  C.inv_dx1 = A.inv_dx1 * ialpha;
  C.inv_dxn1 = A.inv_dxn1 * ialpha;
  C.scl1 = A.scl ? A.scl[0] : 0.f;
  C.scln = A.scl ? A.scl[n - 1] : 0.f;
  Geo<float> g[3];
#pragma unroll
  for (int t = 0; t < 3; ++t) g[t] = geo_at(A, o - 1 + t, alpha, ialpha);
  return general_cell(w, o, C, g, p);
}

// Warp-aggregated append to the worklist; every lane of the warp calls it.
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
// cells of a y-sweep tile staged in shared memory: 16 rows (4 warps of 4) x 32 columns
constexpr int kYTileCells = 16 * 32;

// Line L and position o of a worklist entry (line-1)*n + (position-1).
__device__ __forceinline__ void entry_cell(const SweepArgs& A, uint32_t ent, int& L, int& o) {
  L = (int)(ent / (uint32_t)A.n) + 1;
  o = (int)(ent % (uint32_t)A.n) + 1;
}

// The value of line cell (L, o) through the full rules.
template <int DIR, bool COH>
__device__ __forceinline__ OutCell<float> general_value(const SweepArgs& A, int L, int o) {
  const int n = A.n;
  float alpha = 1.f, ialpha = 1.f;
  if (DIR == 0 && A.lscale != nullptr) {
    const float2 s = A.lscale[L - 1];
    alpha = s.x;
    ialpha = s.y;
  }
  const EdgeVals<float> eL = o == 1 ? edge_vals(A, L, 0) : EdgeVals<float>{0.f, 0.f, 0.f};
  const EdgeVals<float> eR = o == n ? edge_vals(A, L, 1) : EdgeVals<float>{0.f, 0.f, 0.f};
  return general_path<DIR, COH>(A, L, o, alpha, ialpha, eL, eR);
}

// One listed cell through the full rules into a y-sweep tile in shared
// memory (kYTileCells per field, row-major 32 wide; row0/col0: the tile's
// first row and column, 0-based); returns true when the value is finite.
template <bool COH>
__device__ __noinline__ bool general_to_tile(const SweepArgs& A, uint32_t ent, float* tile, int row0, int col0) {
  int L, o;
  entry_cell(A, ent, L, o);
  const OutCell<float> r = general_value<1, COH>(A, L, o);
  const int k = (o - 1 - row0) * 32 + (L - 1 - col0);
  tile[k] = r.s;
  tile[kYTileCells + k] = r.v;      // x velocity (tangential in the y-sweep)
  tile[2 * kYTileCells + k] = r.u;  // y velocity (normal)
  return isfinite(r.s + r.u + r.v);
}

// One listed cell through the full rules, written with its max-wave update.
template <int DIR, bool COH>
__device__ __noinline__ void general_store(const SweepArgs& A, uint32_t ent) {
  int L, o;
  entry_cell(A, ent, L, o);
  const size_t q = cidx<DIR>(L, o, A.pitch);
  // every global read this cell needs goes out before the compute
  const float dq = __ldg(A.dep + q);
  float hm = 0.f, vm = 0.f;
  if (A.hmax) {
    hm = ld_state<COH>(A.hmax + q);
    vm = ld_state<COH>(A.velmax + q);
  }
  const OutCell<float> r = general_value<DIR, COH>(A, L, o);
  const float xo = DIR == 0 ? r.u : r.v;
  const float yo = DIR == 0 ? r.v : r.u;
  A.srf_o[q] = r.s;
  A.xu_o[q] = xo;
  A.yv_o[q] = yo;
  if (A.hmax) {  // max-wave update (cliffs_main.f:347-355)
    A.hmax[q] = fmaxf(hm, eta_of(r.s, dq));
    A.velmax[q] = fmaxf(vm, fma_rn(xo, xo, mul_rn(yo, yo)));
  }
  if (!isfinite(r.s + xo + yo)) atomicOr(A.status, ST_NAN);
}

// The cells of a thread that the plain update does not cover (bits of
// `rest`, cells i0+r of line L): line ends, shorelines, dry cells,
// supercritical flow.  d, e (eta), u (normal), v (tangential), H, c are the
// window at positions i0-1 .. i0+4; wet as computed for the plain update,
// without the line's range, which is applied here (in place).  A line end next to a wet cell
// takes the open or forced edge update in place; a dry cell at the zero state
// between dry neighbours stays as it is; every other cell is returned for the
// general path (bit r).
__device__ __forceinline__ unsigned rest_cells(const SweepArgs& A, int L, int i0, unsigned rest, const float (&d)[6],
                                               const float (&e)[6], const float (&u)[6], const float (&v)[6],
                                               const float (&H)[6], const float (&c)[6], bool (&wet)[6],
                                               float ialpha, float (&os)[kCellsPerThread],
                                               float (&ou)[kCellsPerThread], float (&ov)[kCellsPerThread]) {
  const int n = A.n;
  const Phys<float>& p = A.ph;
  unsigned need = 0u;
#pragma unroll
  for (int w = 0; w < 6; ++w) wet[w] = wet[w] && i0 - 1 + w >= 1 && i0 - 1 + w <= n;  // positions 1..n only
#pragma unroll
  for (int r = 0; r < kCellsPerThread; ++r) {
    if (!((rest >> r) & 1u)) continue;
    const int k = i0 + r;
    const int w = r + 1;
    if ((r == 0 && k == 1 && wet[w] && wet[w + 1]) ||
        (r == kCellsPerThread - 1 && k == n && wet[w - 1] && wet[w])) {
      // line end next to a wet cell: no flooding reaches it; the open or
      // forced edge update (cliffs.f:287-329), or the cell as it is.  Only
      // the thread's first and last cell can take it here (one copy each in
      // the unrolled loop); other line ends go to the general path.
      const EdgeVals<float> ev = edge_vals(A, L, k == 1 ? 0 : 1);
      if (ev.eta + d[w] > p.ground) {
        const CellState<float> j{u[w], c[w], e[w], d[w], v[w], H[w]};
        float cn;
        if (k == 1) {
          const CellState<float> b{u[w + 1], c[w + 1], e[w + 1], d[w + 1], v[w + 1], H[w + 1]};
          edge_left(j, b, ev, A.inv_dx1 * ialpha, A.scl ? A.scl[0] : 0.f, p, cn, ou[r], ov[r], os[r]);
        } else {
          const CellState<float> a{u[w - 1], c[w - 1], e[w - 1], d[w - 1], v[w - 1], H[w - 1]};
          edge_right(a, j, ev, A.inv_dxn1 * ialpha, A.scl ? A.scl[n - 1] : 0.f, p, cn, ou[r], ov[r], os[r]);
        }
      }
    } else if (!(!wet[w] && !wet[w - 1] && !wet[w + 1] && H[w] == 0.f && u[w] == 0.f && v[w] == 0.f)) {
      need |= 1u << r;
    }
    // else: dry, zero state: unchanged whether or not the line holds water
  }
  return need;
}

// The plain VTCS-2 interior update of the cells i0..i0+3 from their window
// (positions i0-1 .. i0+4: d depth, e eta, u normal and v tangential velocity,
// H total depth, c celerity, wet = H > ground; FP/FQ the face fluxes between
// window cells w and w+1; sup: a supercritical cell in the window).  Every
// cell takes the update straight through (no per-cell branches); it is kept
// in os/ou/ov where the cell is interior, wet between wet neighbours, and no
// transcritical point can occur (a transcritical point needs a supercritical
// neighbour).  Returns the cells that are not plain interior cells (bit r);
// cour gets the max of (|u|+c) dt/(dx(m-1)+dx(m)) over the 4 cells.  FLAT:
// the line is known to have uniform spacing and no metric term (the caller
// checked A.geo_uniform and A.scl == nullptr), so neither is read per cell.
template <bool SHARED_ARGS, bool FLAT = false>
__device__ __forceinline__ unsigned plain_cells(const SweepArgs& A, int i0, bool sup, const float (&d)[6],
                                                const float (&e)[6], const float (&u)[6], const float (&v)[6],
                                                const float (&H)[6], const float (&c)[6], const bool (&wet)[6],
                                                const float (&FP)[5], const float (&FQ)[5], float alpha,
                                                float ialpha, float (&os)[kCellsPerThread],
                                                float (&ou)[kCellsPerThread], float (&ov)[kCellsPerThread],
                                                float& cour) {
  const int n = A.n;
  const Phys<float>& p = A.ph;
  unsigned rest = 0u;  // bit r: cell i0+r is not a plain interior cell
  const Geo<float> g0{A.geo0.x * ialpha, A.geo0.y * ialpha, A.geo0.z * ialpha, A.geo0.w * alpha, 0.f};
#pragma unroll
  for (int r = 0; r < kCellsPerThread; ++r) {
    const int k = i0 + r;
    const int w = r + 1;
    const bool plain = !sup && k >= 2 && k <= n - 1 && wet[w - 1] && wet[w] && wet[w + 1];
    const CellState<float> a{u[w - 1], c[w - 1], e[w - 1], d[w - 1], v[w - 1], H[w - 1]};
    const CellState<float> j{u[w], c[w], e[w], d[w], v[w], H[w]};
    const CellState<float> b{u[w + 1], c[w + 1], e[w + 1], d[w + 1], v[w + 1], H[w + 1]};
    float cn;
    const Geo<float> gk =
        FLAT ? g0 : SHARED_ARGS ? geo_at(A, k, alpha, ialpha) : geo_plain(A, min(k, n), g0, alpha, ialpha);
    const OutCell<float> o =
        interior_update<float, false, !FLAT>(a, j, b, FP[w - 1], FQ[w - 1], FP[w], FQ[w], gk, p, &cn);
    // (|u|+c) dt / ((dx(m-1)+dx(m))/2) = 2 (|u|+c) dtx, of the state read
    cour = fmaxf(cour, (fabsf(u[w]) + c[w]) * gk.dtx);
    os[r] = plain ? o.s : os[r];
    ou[r] = plain ? o.u : ou[r];
    ov[r] = plain ? o.v : ov[r];
    if (!plain && k <= n) rest |= 1u << r;
  }
  return rest;
}

template <int DIR, bool LOCAL, bool COH, bool TAIL = true, bool SHARED_ARGS = false, bool MAXOUT = true,
          bool FLAT = false, bool YSMEM = false>
__device__ __forceinline__ void sweep_cells(const SweepArgs& A, int L, int i0, bool active, size_t q0,
                                            float (&d)[6], float (&e)[6], float (&u)[6], float (&v)[6],
                                            float (&hm)[kCellsPerThread], float (&vm)[kCellsPerThread],
                                            uint32_t* s_list, unsigned* s_n, float* s_out = nullptr);

// LOCAL: the block finishes its own listed cells after its fast cells (a
// block-local list in shared memory); otherwise they go to the global
// worklist for general_kernel.
// One tile of a sweep: the block's cells at block coordinates (bx, by) of the
// sweep's grid (x: (columns / (4 * blockDim.x), rows); y: (rows / (4 * warps),
// columns / 32)).  The whole block calls it.  MAXOUT = false leaves out the
// max-wave update of the outputs (A.hmax is then ignored).  FLAT: uniform
// spacing and no metric term (plain_cells).
template <int DIR, bool LOCAL, bool COH, bool SHARED_ARGS = false, bool MAXOUT = true, bool FLAT = false>
__device__ __forceinline__ void sweep_tile(const SweepArgs& A, int bx, int by) {
  __shared__ uint32_t s_list[LOCAL ? 256 * 4 : 1];
  __shared__ unsigned s_n;
  if (LOCAL) {
    if (threadIdx.x == 0) s_n = 0u;
    __syncthreads();
  } else if (bx == 0 && by == 0 && threadIdx.x == 0) {
    *A.count_next = 0u;
  }
  const int lane = threadIdx.x & 31;
  const int n = A.n;
  int L, i0;  // line, first position (1-based)
  if (DIR == 0) {
    L = by + 1;
    i0 = (bx * (int)blockDim.x + (int)threadIdx.x) * kCellsPerThread + 1;
  } else {
    L = by * 32 + lane + 1;
    i0 = (bx * (int)(blockDim.x >> 5) + (int)(threadIdx.x >> 5)) * kCellsPerThread + 1;
  }
  const bool active = L <= A.nlines && i0 <= n;
  // window w[0..5] = positions i0-1 .. i0+4 (u normal, v tangential); e
  // holds the surface state as loaded, then eta
  float d[6], e[6], u[6], v[6];
  float hm[kCellsPerThread], vm[kCellsPerThread];
  size_t q0 = 0;
  if (DIR == 0) {
    q0 = cidx<0>(min(L, A.nlines), i0, A.pitch);
    // the halo cells of the warp's ends first, so that their loads do not
    // wait behind the shuffles of the window
    const bool hl = active && lane == 0 && i0 > 1, hr = active && lane == 31 && i0 + 4 <= n;
    float hd = 0.f, he = 0.f, hu = 0.f, hv = 0.f;
    if (hl || hr) {
      const size_t qh = hl ? q0 - 1 : q0 + 4;
      hd = __ldg(A.dep + qh);
      he = ld_state<COH>(A.srf + qh);
      hu = ld_state<COH>(A.xu + qh);
      hv = ld_state<COH>(A.yv + qh);
    }
    float4 D4 = make_float4(0, 0, 0, 0), E4 = D4, X4 = D4, Y4 = D4, H4 = D4, V4 = D4;
    if (active) {
      D4 = __ldg(reinterpret_cast<const float4*>(A.dep + q0));
      E4 = ld_state4<COH>(A.srf + q0);
      X4 = ld_state4<COH>(A.xu + q0);
      Y4 = ld_state4<COH>(A.yv + q0);
      if (MAXOUT && A.hmax) {
        H4 = ld_state4<COH>(A.hmax + q0);
        V4 = ld_state4<COH>(A.velmax + q0);
      }
      if (A.hmax_in) {
        // the previous step's end state into the max-wave fields
        // (cliffs_main.f:347-355), before this sweep replaces it
        float4 HI = ld_state4<COH>(A.hmax_in + q0), VI = ld_state4<COH>(A.velmax_in + q0);
        HI.x = fmaxf(HI.x, eta_of(E4.x, D4.x));
        HI.y = fmaxf(HI.y, eta_of(E4.y, D4.y));
        HI.z = fmaxf(HI.z, eta_of(E4.z, D4.z));
        HI.w = fmaxf(HI.w, eta_of(E4.w, D4.w));
        VI.x = fmaxf(VI.x, fma_rn(X4.x, X4.x, mul_rn(Y4.x, Y4.x)));
        VI.y = fmaxf(VI.y, fma_rn(X4.y, X4.y, mul_rn(Y4.y, Y4.y)));
        VI.z = fmaxf(VI.z, fma_rn(X4.z, X4.z, mul_rn(Y4.z, Y4.z)));
        VI.w = fmaxf(VI.w, fma_rn(X4.w, X4.w, mul_rn(Y4.w, Y4.w)));
        *reinterpret_cast<float4*>(A.hmax_in + q0) = HI;
        *reinterpret_cast<float4*>(A.velmax_in + q0) = VI;
      }
    }
    d[1] = D4.x; d[2] = D4.y; d[3] = D4.z; d[4] = D4.w;
    e[1] = E4.x; e[2] = E4.y; e[3] = E4.z; e[4] = E4.w;
    u[1] = X4.x; u[2] = X4.y; u[3] = X4.z; u[4] = X4.w;
    v[1] = Y4.x; v[2] = Y4.y; v[3] = Y4.z; v[4] = Y4.w;
    hm[0] = H4.x; hm[1] = H4.y; hm[2] = H4.z; hm[3] = H4.w;
    vm[0] = V4.x; vm[1] = V4.y; vm[2] = V4.z; vm[3] = V4.w;
    d[0] = __shfl_up_sync(0xffffffffu, D4.w, 1);
    e[0] = __shfl_up_sync(0xffffffffu, E4.w, 1);
    u[0] = __shfl_up_sync(0xffffffffu, X4.w, 1);
    v[0] = __shfl_up_sync(0xffffffffu, Y4.w, 1);
    d[5] = __shfl_down_sync(0xffffffffu, D4.x, 1);
    e[5] = __shfl_down_sync(0xffffffffu, E4.x, 1);
    u[5] = __shfl_down_sync(0xffffffffu, X4.x, 1);
    v[5] = __shfl_down_sync(0xffffffffu, Y4.x, 1);
    if (hl) {
      d[0] = hd;
      e[0] = he;
      u[0] = hu;
      v[0] = hv;
    }
    if (hr) {
      d[5] = hd;
      e[5] = he;
      u[5] = hu;
      v[5] = hv;
    }
  } else {
#pragma unroll
    for (int w = 0; w < 6; ++w) {
      const int k = min(max(i0 - 1 + w, 1), n);
      const size_t q = cidx<1>(min(L, A.nlines), k, A.pitch);
      d[w] = e[w] = u[w] = v[w] = 0.f;
      if (active) {
        d[w] = __ldg(A.dep + q);
        e[w] = ld_state<COH>(A.srf + q);
        v[w] = ld_state<COH>(A.xu + q);  // tangential in the y-sweep
        u[w] = ld_state<COH>(A.yv + q);  // normal
      }
    }
#pragma unroll
    for (int r = 0; r < kCellsPerThread; ++r) {
      hm[r] = vm[r] = 0.f;
      const int k = min(i0 + r, n);
      if (MAXOUT && active && A.hmax) {
        const size_t q = cidx<1>(L, k, A.pitch);
        hm[r] = ld_state<COH>(A.hmax + q);
        vm[r] = ld_state<COH>(A.velmax + q);
      }
    }
  }
  sweep_cells<DIR, LOCAL, COH, true, SHARED_ARGS, MAXOUT, FLAT>(A, L, i0, active, q0, d, e, u, v, hm, vm, s_list,
                                                                &s_n);
}

// The cells i0..i0+3 of line L from their loaded window: d depth, e surface
// state, u normal and v tangential velocity at positions i0-1 .. i0+4, hm/vm
// the max-wave values of the 4 cells (when fused).  Updates and stores them;
// cells that need the full wet/dry rules go to the block's list s_list
// (LOCAL: finished by the whole block after a __syncthreads) or to the
// global worklist.  q0 is the first cell's index (x-sweep).  The whole block
// calls it.  TAIL = false leaves the block's list to the caller, who must
// finish it after a barrier (the fast stores come first).  SHARED_ARGS: A
// lives in shared memory (the batched kernels), where every field read is a
// load; the geometry is then read per cell instead of held in registers for
// the whole line, which measured 14 % faster there (fewer spills).  YSMEM
// (y-sweep): the outputs go to a shared-memory tile instead of global memory,
// s_out[f * kYTileCells + r * 32] for field f (surface state, x velocity, y
// velocity) and cell i0 + r (s_out points at the thread's first cell); the
// caller stores the tile.
template <int DIR, bool LOCAL, bool COH, bool TAIL, bool SHARED_ARGS, bool MAXOUT, bool FLAT, bool YSMEM>
__device__ __forceinline__ void sweep_cells(const SweepArgs& A, int L, int i0, bool active, size_t q0,
                                            float (&d)[6], float (&e)[6], float (&u)[6], float (&v)[6],
                                            float (&hm)[kCellsPerThread], float (&vm)[kCellsPerThread],
                                            uint32_t* s_list, unsigned* s_n, float* s_out) {
  const int n = A.n;
  const bool swept = active && L >= A.lo && L <= A.hi;
  const Phys<float>& p = A.ph;
  // os: new surface state of cells i0..i0+3, initially the state as loaded
  float os[kCellsPerThread], ou[kCellsPerThread], ov[kCellsPerThread];
#pragma unroll
  for (int r = 0; r < kCellsPerThread; ++r) {
    os[r] = e[r + 1];
    ou[r] = u[r + 1];
    ov[r] = v[r + 1];
  }
  float H[6];
#pragma unroll
  for (int w = 0; w < 6; ++w) {  // surface state -> (eta, H); the stored form stays exact in one of them
    H[w] = e[w] + fmaxf(d[w], 0.f);  // depth_of and eta_of without a branch
    e[w] = e[w] - fminf(d[w], 0.f);
  }
  unsigned need = 0u;  // bit r: cell i0+r goes to the general path
  float cour = 0.f;    // half the largest Courant number of the thread's cells
  if (swept) {  // lines not swept are copied through
    float alpha = 1.f, ialpha = 1.f;
    if (DIR == 0 && A.lscale != nullptr) {
      const float2 s = A.lscale[L - 1];
      alpha = s.x;
      ialpha = s.y;
    }
    bool wet[6];
    float c[6];
    bool sup = false;  // a supercritical cell (|u| > c) in the window
#pragma unroll
    for (int w = 0; w < 6; ++w) {
      // in range or not: the window of a cell that can take the plain update
      // (2 <= k <= n-1) is; the rare branch below applies the range
      wet[w] = H[w] > p.ground;
      c[w] = fsqrt_pos(p.g * fmaxf(H[w], p.ground));
      sup = sup || fabsf(u[w]) > c[w];
    }
    float FP[5], FQ[5];  // face fluxes between window cells w and w+1
#pragma unroll
    for (int f = 0; f < 5; ++f) face_flux(u[f], c[f], e[f], u[f + 1], c[f + 1], e[f + 1], p, FP[f], FQ[f]);
    const unsigned rest = plain_cells<SHARED_ARGS, FLAT>(A, i0, sup, d, e, u, v, H, c, wet, FP, FQ, alpha, ialpha, os, ou,
                                                   ov, cour);
    if (rest) need = rest_cells(A, L, i0, rest, d, e, u, v, H, c, wet, ialpha, os, ou, ov);
  }
  if (LOCAL) {
#pragma unroll
    for (int r = 0; r < kCellsPerThread; ++r)
      if (active && ((need >> r) & 1u))
        s_list[atomicAdd(s_n, 1u)] = (uint32_t)(L - 1) * (uint32_t)n + (uint32_t)(i0 + r - 1);
  } else {
#pragma unroll
    for (int r = 0; r < kCellsPerThread; ++r)
      enqueue(A, active && ((need >> r) & 1u), (uint32_t)(L - 1) * (uint32_t)n + (uint32_t)(i0 + r - 1));
  }
  bool bad = false;
  float xo[kCellsPerThread], yo[kCellsPerThread];
#pragma unroll
  for (int r = 0; r < kCellsPerThread; ++r) {
    if (!active) break;
    xo[r] = DIR == 0 ? ou[r] : ov[r];
    yo[r] = DIR == 0 ? ov[r] : ou[r];
    const bool done = i0 + r <= n && !((need >> r) & 1u);
    if (done) bad |= !isfinite(os[r] + xo[r] + yo[r]);
    if (MAXOUT && A.hmax && done) {  // max-wave update (cliffs_main.f:347-355)
      hm[r] = fmaxf(hm[r], eta_of(os[r], d[r + 1]));
      vm[r] = fmaxf(vm[r], fma_rn(xo[r], xo[r], mul_rn(yo[r], yo[r])));
    }
  }
  if (!active) {
    // nothing to store
  } else if (DIR == 0) {
    // whole float4s: the row padding beyond nx takes the values of no cell
    *reinterpret_cast<float4*>(A.srf_o + q0) = make_float4(os[0], os[1], os[2], os[3]);
    *reinterpret_cast<float4*>(A.xu_o + q0) = make_float4(xo[0], xo[1], xo[2], xo[3]);
    *reinterpret_cast<float4*>(A.yv_o + q0) = make_float4(yo[0], yo[1], yo[2], yo[3]);
    if (MAXOUT && A.hmax) {
      *reinterpret_cast<float4*>(A.hmax + q0) = make_float4(hm[0], hm[1], hm[2], hm[3]);
      *reinterpret_cast<float4*>(A.velmax + q0) = make_float4(vm[0], vm[1], vm[2], vm[3]);
    }
  } else if (YSMEM) {
    // every row of the tile: rows past the grid are clipped by the tile store
#pragma unroll
    for (int r = 0; r < kCellsPerThread; ++r) {
      s_out[r * 32] = os[r];
      s_out[kYTileCells + r * 32] = xo[r];
      s_out[2 * kYTileCells + r * 32] = yo[r];
    }
  } else {
#pragma unroll
    for (int r = 0; r < kCellsPerThread; ++r) {
      const int k = i0 + r;
      if (k > n) break;
      const size_t q = cidx<1>(L, k, A.pitch);
      A.srf_o[q] = os[r];
      A.xu_o[q] = xo[r];
      A.yv_o[q] = yo[r];
      if (MAXOUT && A.hmax) {
        A.hmax[q] = hm[r];
        A.velmax[q] = vm[r];
      }
    }
  }
  if (bad) atomicOr(A.status, ST_NAN);
  // Courant check: a warp vote, and in the rare warp with a number above 1
  // a warp max reduction and one atomic (the reference fixes dt and checks
  // nothing; VTCS-2 is stable for Courant numbers up to 1)
  if (__any_sync(0xffffffffu, cour > 0.5f)) {
    const unsigned m = __reduce_max_sync(0xffffffffu, __float_as_uint(2.f * cour));
    if ((threadIdx.x & 31) == 0) {
      atomicOr(A.status, ST_CFL);
      atomicMax(A.status + 1, m);
    }
  }
  if (LOCAL && TAIL) {
    __syncthreads();  // the block's fast values are stored; its listed cells overwrite theirs
    const unsigned cnt = *s_n;
    for (unsigned t = threadIdx.x; t < cnt; t += blockDim.x) general_store<DIR, COH>(A, s_list[t]);
  }
}

// Launched with programmatic stream serialization, consecutive sweeps
// overlap their launch: this grid lets the next one be scheduled once all of
// its own blocks have started, and waits for the previous grid to complete
// (its stores visible) before any load or store of the state.  Without the
// launch attribute both instructions are no-ops.
// MAXOUT = false: the variant without the max-wave update of the outputs
// (the y-sweep of a two-dimensional step, whose end state the next x-sweep
// folds in through hmax_in).  FLAT = true: a grid whose lines of this
// direction have uniform spacing and no metric term (A.geo_uniform,
// A.scl == nullptr: every x-sweep of a grid with uniform dx, every y-sweep
// of a Cartesian grid with uniform dy).
template <int DIR, bool LOCAL, bool MAXOUT = true, bool FLAT = false>
__global__ void __launch_bounds__(256, 4) fast_kernel(const SweepArgs A) {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  asm volatile("griddepcontrol.wait;" ::: "memory");
  if (DIR == 0 || !LOCAL) {  // the worklist variant: grid (bands, column groups) for the y-sweep
    sweep_tile<DIR, LOCAL, false, false, MAXOUT, FLAT>(A, blockIdx.x, blockIdx.y);
  } else {
    // y tiles in bands of 4 * warps rows, the last band first: the x-sweep
    // before this one wrote its rows first to last, so the bands it wrote
    // last are read while they are still in L2; this sweep in turn writes the
    // first bands last, which the next x-sweep reads first
    sweep_tile<DIR, LOCAL, false, false, MAXOUT, FLAT>(A, (int)(gridDim.y - 1 - blockIdx.y), blockIdx.x);
  }
}

// One thread per listed cell: the full wet/dry rules over its +-3 window.
template <int DIR>
__global__ void __launch_bounds__(128) general_kernel(const SweepArgs A) {
  const uint32_t cnt = *A.count;
  for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < cnt; t += gridDim.x * blockDim.x) {
    general_store<DIR, false>(A, A.list[t]);
  }
}

// Forcing at the line ends of one sweep for the current step: edge1/edge2
// lerped from the boundary records in FP64 (cliffs_main.f:318-324 for the
// x-sweep, 333-339 for the y-sweep), stored as 6 floats per line.  recA/recB
// are the records of the low and high edge, (len,3,nt); irec is 1-based with
// tinput(irec-1) <= t < tinput(irec); cc the weight of record irec-1.  cn is
// the normal velocity component (iu-1 in the reference), ct the tangential.
__device__ __forceinline__ void edges_line(int L, int len, const double* __restrict__ recA,
                                           const double* __restrict__ recB, int irec, double cc, int cn, int ct,
                                           float* out) {
  const size_t r0 = (size_t)(irec - 2) * 3 * (size_t)len;
  const size_t r1 = (size_t)(irec - 1) * 3 * (size_t)len;
  const int comp[3] = {cn, ct, 2};
#pragma unroll
  for (int side = 0; side < 2; ++side) {
    const double* F = side == 0 ? recA : recB;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      float v = 0.f;
      if (F) {
        const size_t b = (size_t)L + (size_t)comp[k] * (size_t)len;
        v = (float)(F[b + r0] * cc + F[b + r1] * (1.0 - cc));
      }
      out[(size_t)L * 6 + side * 3 + k] = v;
    }
  }
}

__global__ void edges_kernel(int nlines, int len, const double* __restrict__ recA, const double* __restrict__ recB,
                             int irec, double cc, int cn, int ct, float* out) {
  const int L = blockIdx.x * blockDim.x + threadIdx.x;
  if (L >= nlines) return;
  edges_line(L, len, recA, recB, irec, cc, cn, ct, out);
}

// The edge tables of k forced steps at once, for replay from a graph: step s
// of the x-sweep (ny lines, west/east records) into ring_x + s*6*ny, of the
// y-sweep (nx lines, south/north) into ring_y + s*6*nx, with record irec[s]
// and weight cc[s] as the time loop's cursor gives them.  A thread per line
// and step; the values are those edges_kernel writes.
__global__ void edges_ring_kernel(int k, int nx, int ny, const double* __restrict__ fw, const double* __restrict__ fe,
                                  const double* __restrict__ fs, const double* __restrict__ fn,
                                  const int* __restrict__ irec, const double* __restrict__ cc, float* ring_x,
                                  float* ring_y) {
  const int per = nx + ny;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)per * k) return;
  const int s = (int)(t / per), L = (int)(t % per);
  if (L < ny)
    edges_line(L, ny, fw, fe, irec[s], cc[s], 0, 1, ring_x + (size_t)s * 6 * ny);
  else
    edges_line(L - ny, nx, fs, fn, irec[s], cc[s], 1, 0, ring_y + (size_t)s * 6 * nx);
}

}  // namespace cliffs
