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
#include <type_traits>

#include "march.cuh"
#include "tma.cuh"

namespace cliffs {

constexpr int kChunk = 8;        // cells per line per pipeline chunk
constexpr int kWarpsPerCta = 4;
constexpr int kPlane = 32 * kChunk;  // floats in one plane (32 lines x 8 cells)

// Pipeline depth and shared memory per warp of each sweep direction.
template <int DIR>
struct SweepCfg;
template <>
struct SweepCfg<0> {  // x-sweep: lines are rows, TMA transposes both ways
  static constexpr int NST = 3;
  static constexpr int PLANES = 4;  // dep, eta, xvel, yvel
  static constexpr int OUTB = 2;
};
template <>
struct SweepCfg<1> {  // y-sweep: lines are columns, rows of a chunk are coalesced
  static constexpr int NST = 3;
  static constexpr int PLANES = 6;  // + hmax, velmax of the chunk's output rows
  static constexpr int OUTB = 0;
};
template <int DIR>
__host__ __device__ constexpr int warp_smem_bytes() {
  return (SweepCfg<DIR>::NST * SweepCfg<DIR>::PLANES + SweepCfg<DIR>::OUTB * 3) * kPlane * 4 + 128;
}

struct SweepParams {
  CUtensorMap tm_in[6];   // dep, eta, xvel, yvel of the input state; hmax, velmax
  CUtensorMap tm_out[3];  // eta, xvel, yvel of the output state (x-sweep)
  int pitch;
  int n;       // line length (nx for the x-sweep, ny for the y-sweep)
  int nlines;  // number of lines (ny for x, nx for y)
  int lo, hi;  // swept lines, 1-based; other lines are copied through
  int seg;     // output cells per warp work item, multiple of 32
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
  int geo_uniform;    // all interior positions share geo0 (uniform spacing)
  float4 geo0;
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

enum : unsigned { ST_NAN = 1u, ST_TIMEOUT = 2u };
constexpr int kWaitLimit = 1 << 22;

template <int DIR>
__device__ __forceinline__ size_t cell_index(int L, int k, int pitch) {
  // DIR 0: line L is row j, position k is column i; DIR 1: line L is column i
  return DIR == 0 ? (size_t)(L - 1) * (size_t)pitch + (size_t)(k - 1)
                  : (size_t)(k - 1) * (size_t)pitch + (size_t)(L - 1);
}

// One warp per work item: 32 consecutive lines x one segment of `seg` output
// cells.  The segment plus an 8-cell halo chunk on each side streams through a
// per-warp ring of shared-memory stages filled by TMA (one 2-D box per field
// and chunk: 8 cells x 32 lines); each lane marches its own line through it
// (cliffs.f:17-346 via LineMarch).  The x-sweep writes its output through a
// second ring and TMA stores (the transposition back to rows); the y-sweep
// stores straight from registers, coalesced across lanes.
template <int DIR>
__global__ void __launch_bounds__(128) sweep_kernel(const __grid_constant__ SweepParams P) {
  constexpr int NST = SweepCfg<DIR>::NST;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31;
  const int wic = threadIdx.x >> 5;
  const int gw = blockIdx.x * kWarpsPerCta + wic;
  const int nlb = (P.nlines + 31) >> 5;
  const int nseg = (P.n + P.seg - 1) / P.seg;
  if (gw >= nlb * nseg) return;  // warp-uniform
  unsigned char* wbase = smem_raw + (size_t)wic * warp_smem_bytes<DIR>();
  float* inb = reinterpret_cast<float*>(wbase);
  float* outb = inb + NST * SweepCfg<DIR>::PLANES * kPlane;
  uint64_t* bar = reinterpret_cast<uint64_t*>(wbase + warp_smem_bytes<DIR>() - 128);

  const int lb = gw / nseg;
  const int sg = gw - lb * nseg;
  const int L = (lb << 5) + lane + 1;
  const int n = P.n;
  const bool active = L <= P.nlines;
  const bool swept = active && L >= P.lo && L <= P.hi;
  const int o0 = sg * P.seg + 1;
  const int o1 = min(o0 + P.seg - 1, n);
  const int NQ = (o1 - o0) / kChunk + 3;  // chunks: halo, segment, halo (+ flush)
  const int kb = max(1, o0 - 3);
  const int ke = o1 + 3;

  constexpr int NPL = SweepCfg<DIR>::PLANES;
  const bool maxw = DIR == 1 && P.hmax != nullptr;
  auto issue = [&](int q) {  // lane 0: TMA the input planes of chunk q
    const int s = q % NST;
    const int p0 = o0 - kChunk + kChunk * q;  // first position of the chunk (1-based)
    const int npl = maxw ? 6 : 4;
    mbar_expect_tx(&bar[s], npl * kPlane * 4);
#pragma unroll
    for (int f = 0; f < 4; ++f) {
      float* dst = inb + (s * NPL + f) * kPlane;
      if (DIR == 0)
        tma_load_2d(dst, &P.tm_in[f], &bar[s], p0 - 1, lb * 32);
      else
        tma_load_2d(dst, &P.tm_in[f], &bar[s], lb * 32, p0 - 1);
    }
    if (maxw) {  // max-wave rows of the outputs this chunk produces: p0-3 .. p0+4
#pragma unroll
      for (int f = 4; f < 6; ++f)
        tma_load_2d(inb + (s * NPL + f) * kPlane, &P.tm_in[f], &bar[s], lb * 32, p0 - 4);
    }
  };
  if (lane == 0) {
    for (int s = 0; s < NST; ++s) mbar_init(&bar[s], 1);
    fence_mbar_init();
    for (int q = 0; q < NST && q < NQ; ++q) issue(q);
  }
  __syncwarp();

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

  uint32_t acc_bits = 0;
  bool bad = false;
  float4 rb[4];                          // x-sweep: 4 raw cells per plane
  float oacc0[4], oacc1[4], oacc2[4];    // x-sweep: 4 outputs per plane
#pragma unroll
  for (int t = 0; t < 4; ++t) oacc0[t] = oacc1[t] = oacc2[t] = 0.f;
  const uint32_t* myw = P.bm_in + (size_t)(min(L, P.nlines) - 1) * (size_t)P.ld_in;

  for (int q = 0; q < NQ; ++q) {
    const int s = q % NST;
    const bool ok = mbar_wait_bounded(&bar[s], (uint32_t)((q / NST) & 1), kWaitLimit);
    if (!__all_sync(0xffffffffu, ok)) {
      if (lane == 0) atomicOr(P.status, ST_TIMEOUT);
      // let the copies already issued land before the shared memory goes away
      for (int r = q; r < NQ && r < q + NST; ++r)
        mbar_wait_bounded(&bar[r % NST], (uint32_t)((r / NST) & 1), kWaitLimit);
      if (DIR == 0 && lane == 0) bulk_wait<0>();
      return;
    }
    const float* st = inb + s * NPL * kPlane;
    const int p0 = o0 - kChunk + kChunk * q;

    // A chunk whose cells k-3..k are wet on every swept line takes the
    // flood-free path; the wetness comes from the bitmap the previous sweep
    // wrote with the same predicate (d + eta > ground).
    bool fast = false;
    if (p0 >= 5 && p0 + kChunk - 1 <= n - 1 && p0 >= kb && p0 + kChunk - 1 <= ke) {
      bool lf = true;
      if (swept) {
        const int a = p0 - 4;  // 0-based bit of position p0-3
        const int wi = a >> 5, sh = a & 31;
        uint64_t word = myw[wi];
        if (sh + kChunk + 3 > 32) word |= (uint64_t)myw[wi + 1] << 32;
        const uint32_t need = (1u << (kChunk + 3)) - 1u;
        lf = ((uint32_t)(word >> sh) & need) == need;
      }
      fast = __all_sync(0xffffffffu, lf);
    }

    auto body = [&](auto fastc) {
      constexpr bool FAST = decltype(fastc)::value;
#pragma unroll(FAST ? kChunk : 1)
      for (int c = 0; c < kChunk; ++c) {
        const int k = p0 + c;
        if (DIR == 0 && (c & 3) == 0) {
#pragma unroll
          for (int f = 0; f < 4; ++f)
            rb[f] = *reinterpret_cast<const float4*>(st + f * kPlane + lane * kChunk + c);
        }
        if (FAST || (k >= kb && k <= ke)) {  // warp-uniform
          float d, e, xu, yv;
          if (DIR == 0) {
            const int t = c & 3;
            d = t == 0 ? rb[0].x : t == 1 ? rb[0].y : t == 2 ? rb[0].z : rb[0].w;
            e = t == 0 ? rb[1].x : t == 1 ? rb[1].y : t == 2 ? rb[1].z : rb[1].w;
            xu = t == 0 ? rb[2].x : t == 1 ? rb[2].y : t == 2 ? rb[2].z : rb[2].w;
            yv = t == 0 ? rb[3].x : t == 1 ? rb[3].y : t == 2 ? rb[3].z : rb[3].w;
          } else {
            d = st[0 * kPlane + c * 32 + lane];
            e = st[1 * kPlane + c * 32 + lane];
            xu = st[2 * kPlane + c * 32 + lane];
            yv = st[3 * kPlane + c * 32 + lane];
          }
          if (!FAST && k > n) d = e = xu = yv = 0.f;
          const float u = DIR == 0 ? xu : yv;
          const float v = DIR == 0 ? yv : xu;
          Geo<float> g{0.f, 0.f, 0.f, 0.f, 0.f};
          const int m = k - 2;
          if (FAST || (m >= 2 && m <= n - 1)) {
            float4 gg;
            if (P.geo_uniform)
              gg = P.geo0;
            else
              gg = __ldg(P.geo + (m - 1));
            g.inv_fm = gg.x * ialpha;
            g.inv_fp = gg.y * ialpha;
            g.dtx = gg.z * ialpha;
            g.dfpm = gg.w * alpha;
            g.scl = P.scl ? __ldg(P.scl + (m - 1)) : 0.f;
          }
          OutCell<float> oc;
          bool has;
          if (FAST) {
            oc = M.push_fast(d, e, u, v, g);
            has = true;
          } else {
            has = M.push(k, d, e, u, v, g, oc);
          }
          const int o = k - 3;
          if (has && o >= o0 && o <= o1) {  // warp-uniform
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
            const bool wetout = active && (M.rd.d + eo) > P.ph.ground;
            if (active) {
              bad |= !isfinite(eo + xo + yo);
              const size_t q2 = cell_index<DIR>(L, o, P.pitch);
              if (DIR == 1) {
                P.eta_out[q2] = eo;
                P.xu_out[q2] = xo;
                P.yv_out[q2] = yo;
                if (maxw) {  // max-wave update (cliffs_main.f:347-355)
                  if (eo > st[4 * kPlane + c * 32 + lane]) P.hmax[q2] = eo;
                  const float s2 = xo * xo + yo * yo;
                  if (s2 > st[5 * kPlane + c * 32 + lane]) P.velmax[q2] = s2;
                }
              } else if (P.hmax) {
                if (eo > P.hmax[q2]) P.hmax[q2] = eo;
                const float s2 = xo * xo + yo * yo;
                if (s2 > P.velmax[q2]) P.velmax[q2] = s2;
              }
            }
            if (DIR == 0) {
              const int t = (c + 1) & 3;  // (o - o0) & 3
              if (t == 0) { oacc0[0] = eo; oacc1[0] = xo; oacc2[0] = yo; }
              if (t == 1) { oacc0[1] = eo; oacc1[1] = xo; oacc2[1] = yo; }
              if (t == 2) { oacc0[2] = eo; oacc1[2] = xo; oacc2[2] = yo; }
              if (t == 3) { oacc0[3] = eo; oacc1[3] = xo; oacc2[3] = yo; }
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
        if (DIR == 0 && (c == 2 || c == 6)) {
          // output positions o = p0 + c - 3: c == 2 closes the 4..7 half of
          // output chunk q-2 (then stored by TMA), c == 6 the 0..3 half of q-1
          const int qo = c == 2 ? q - 2 : q - 1;
          if (qo >= 0 && o0 + kChunk * qo <= o1) {
            float* ob = outb + (qo & 1) * 3 * kPlane + lane * kChunk + (c == 2 ? 4 : 0);
            *reinterpret_cast<float4*>(ob) = make_float4(oacc0[0], oacc0[1], oacc0[2], oacc0[3]);
            *reinterpret_cast<float4*>(ob + kPlane) = make_float4(oacc1[0], oacc1[1], oacc1[2], oacc1[3]);
            *reinterpret_cast<float4*>(ob + 2 * kPlane) = make_float4(oacc2[0], oacc2[1], oacc2[2], oacc2[3]);
            if (c == 2) {
              fence_proxy_async();
              __syncwarp();
              if (lane == 0) {
                const float* src = outb + (qo & 1) * 3 * kPlane;
                const int x = o0 - 1 + kChunk * qo;
                tma_store_2d(&P.tm_out[0], src, x, lb * 32);
                tma_store_2d(&P.tm_out[1], src + kPlane, x, lb * 32);
                tma_store_2d(&P.tm_out[2], src + 2 * kPlane, x, lb * 32);
                bulk_commit();
                bulk_wait_read<1>();  // the other output buffer is free again
              }
              __syncwarp();
            }
          }
        }
      }
    };
    if (fast)
      body(std::true_type{});
    else
      body(std::false_type{});
    __syncwarp();  // every lane is done with stage s
    if (lane == 0 && q + NST < NQ) issue(q + NST);
  }
  if (DIR == 0 && lane == 0) bulk_wait<0>();
  if (bad) atomicOr(P.status, ST_NAN);
}

}  // namespace cliffs
