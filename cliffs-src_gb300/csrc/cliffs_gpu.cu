// cliffs_gpu.cu -- C ABI implementation (include/cliffs_gpu.h) and the
// auxiliary kernels: state conversion, wetness bitmaps, output conversions,
// gauges, runup, nested-grid feed.
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <atomic>
#include <mutex>
#include <initializer_list>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "../../include/cliffs_gpu.h"
#include "batch.cuh"
#include "staged.cuh"
#include "ytile.cuh"
#include "depth_ssl.cuh"
#include "boundary.cuh"

using namespace cliffs;

namespace {

constexpr double kGrav = 9.800000190734863;   // (double)9.8f, global_modules.f:17
constexpr double kPi = 3.1415927410125732;    // (double)3.1415926536f
constexpr double kEarthR = 6371009.0;
constexpr double kSqr2 = 1.4142135381698608;  // (double)1.41421356f, cliffs.f:34
constexpr float kNan4 = -1.0e32f;             // global_modules.f:18

#define CK(x)                                     \
  do {                                            \
    cudaError_t e_ = (x);                         \
    if (e_ != cudaSuccess) return CLIFFS_ERR_CUDA; \
  } while (0)
// a library status: returned when not CLIFFS_OK
#define RET(x)             \
  do {                     \
    const int r_ = (x);    \
    if (r_) return r_;     \
  } while (0)

struct Nest {
  cliffs_nest_desc d;
  int32_t *WE_ny = nullptr, *SN_nx = nullptr;
  double *WE_cy = nullptr, *SN_cx = nullptr;
  // the footprint of the arrival test: parent columns i1..i2, rows k1..k2
  int32_t i1 = 0, i2 = 0, k1 = 0, k2 = 0;
  int* d_arr = nullptr;  // arrival flag on the device, sticky (the asynchronous feed)
};

// One asynchronous output: a device buffer the conversion kernels write and a
// second stream copies to the caller's host buffers, and the events that
// order the two.
struct OutSlot {
  void* dbuf = nullptr;
  size_t cap = 0;
  cudaEvent_t conv = nullptr, done = nullptr;
  bool used = false;
};
constexpr int kOutSlots = 8;

struct ProfPair {
  cudaEvent_t a, b;
  int dir;
};

PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;

int get_encoder() {
  if (g_encode) return CLIFFS_OK;
  cudaDriverEntryPointQueryResult q;
  void* fn = nullptr;
  if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) !=
          cudaSuccess ||
      q != cudaDriverEntryPointSuccess || !fn)
    return CLIFFS_ERR_CUDA;
  g_encode = (PFN_cuTensorMapEncodeTiled_v12000)fn;
  return CLIFFS_OK;
}

// 2-D FP32 map over an nx x ny field with a row pitch of `pitch` floats and a
// box of bx x by elements; elements outside the field read 0.
int make_map(CUtensorMap* m, const float* base, int nx, int ny, int pitch, int bx, int by) {
  cuuint64_t dims[2] = {(cuuint64_t)nx, (cuuint64_t)ny};
  cuuint64_t strides[1] = {(cuuint64_t)pitch * sizeof(float)};
  cuuint32_t box[2] = {(cuuint32_t)bx, (cuuint32_t)by};
  cuuint32_t es[2] = {1, 1};
  const CUresult r = g_encode(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float*>(base), dims, strides, box,
                              es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                              CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? CLIFFS_OK : CLIFFS_ERR_CUDA;
}

}  // namespace

struct cliffs_ctx {
  // one device allocation holding the per-grid arrays (dep, the state
  // copies, the max-wave fields, geometry, status words, worklist, edge
  // tables, dep64, xfer), carved at 256-byte boundaries: cudaMalloc costs
  // ~50 us per large block, one call for all of them a tenth of that
  char* arena = nullptr;
  int dev = 0;
  int nx = 0, ny = 0, pitch = 0;
  bool xrun = false, yrun = false;
  int ii1 = 1, ii2 = 1, jj1 = 1, jj2 = 1;
  double ground = 0, crough = 0, dt = 0, celmin = 0;
  cudaStream_t own = nullptr, stream = nullptr;
  float* dep = nullptr;
  // surface state (eta where dep >= 0, water depth where dep < 0), u, v; ping-pong
  float *srf[2] = {nullptr, nullptr}, *xu[2] = {nullptr, nullptr}, *yv[2] = {nullptr, nullptr};
  float *hmax = nullptr, *velmax = nullptr;
  int cur = 0;
  int64_t launches = 0;  // kernels this context has launched
  // the caller's FP64 depth on the device (nx*ny, unpadded), for the state
  // conversions, and a staging area of 3*nx*ny doubles for FP64 transfers,
  // allocated at the first transfer and kept
  double* dep64 = nullptr;
  double* xfer = nullptr;
  // a source rising over time (cliffs_gpu_add_source): its full uplift, its
  // duration, the time since it was added and the fraction applied so far
  float* rise_q = nullptr;
  double rise_T = 0, rise_el = 0, rise_w = 0;
  bool rise_on = false;
  float4 *geo_x = nullptr, *geo_y = nullptr;
  float* scl_y = nullptr;
  float2* lscale = nullptr;
  float inv_dx1_x = 0, inv_dxn1_x = 0, inv_dx1_y = 0, inv_dxn1_y = 0;
  // boundary forcing
  int nt = 0;
  std::vector<double> tinput;
  double *fw = nullptr, *fe = nullptr, *fs = nullptr, *fn = nullptr;
  int irec = 0;
  bool feed_on = false, freeze = false;
  // static edges for single sweeps (edge1/edge2 of module MASTER)
  double *edge_s[2] = {nullptr, nullptr};
  bool edges_static = false;
  // per-step forcing at the line ends, 6 floats per line, for each sweep
  float* edge_x = nullptr;
  float* edge_y = nullptr;
  unsigned* status = nullptr;
  double* red = nullptr;  // reduction scratch
  int red_cap = 0;
  std::vector<Nest> nests;
  int* d_flag = nullptr;
  bool have_state = false;
  int blk_x = 128, warps_y = 4;
  // worklist of cells for the general kernel and one counter per sweep parity
  uint32_t* list = nullptr;
  uint32_t* cnt = nullptr;
  unsigned sweeps = 0;  // fast-kernel block shapes (cliffs_gpu_set_tiling)
  bool geo_uni_x = false, geo_uni_y = false;
  float4 geo0_x = {0, 0, 0, 0}, geo0_y = {0, 0, 0, 0};
  // steps of the sweep loop captured in a CUDA graph (cliffs_gpu_step);
  // valid for the tiling and state copy it was captured with
  int graph_k = 16;
  // [0]: the graph of graph_k steps; [1..]: graphs of the shorter tails of
  // step calls (their lengths differ), replaced oldest first
  static constexpr int kPlainGraphs = 4;
  struct PlainGraph {
    cudaGraphExec_t exec = nullptr;
    int len = 0, cur = -1, blk = 0, wy = 0, kind = -1;
    int64_t used = 0;
  } pgraph[kPlainGraphs];
  int64_t pgraph_clock = 0;
  // sweep kernels (cliffs_gpu_set_sweep_kernel): the staged persistent pair
  // needs the y-sweep's tensor maps (one per state copy) and its grid size
  int sweep_kind = CLIFFS_SWEEP_TILED;
  bool staged_ok = false;
  CUtensorMap m_dep, m_srf[2], m_xu[2], m_yv[2], m_hmax, m_velmax;
  // the state copies with a 32 x kYRows box: the tile stores of tile_y_kernel
  // (the y-sweep of the tiled kernels when ytile_ok)
  CUtensorMap m_srf16[2], m_xu16[2], m_yv16[2];
  bool ytile_ok = false;
  int grid_sx = 0, grid_sy = 0;  // resident blocks of staged_x / staged_y
  unsigned long long stage_ns = 2000000000ull;  // limit of one stage wait
  // fast-kernel sweeps launched as programmatic dependents of the previous
  // sweep (CLIFFS_PDL=0 in the environment at context creation turns it off)
  bool pdl = true;
  // max-wave bookkeeping of two-dimensional steps with the tiled kernels: the
  // x-sweep folds in the state the previous step ended with, so the end state
  // of the latest step is pending until the next x-sweep or a max_sync.
  // fresh: the state is not the end of a step (initial, uploaded, a source
  // added, after a single sweep) and is never folded in.
  bool max_pending = false, max_fresh = true;
  // forced steps from a graph: per-step edge tables of graph_k steps (ring),
  // the cursor's record and weight of each step, and the graph itself
  float *ring_x = nullptr, *ring_y = nullptr;
  int32_t* ring_irec = nullptr;
  double* ring_cc = nullptr;
  int ring_k = 0;
  // pinned host slots for the cursor of the next chunks, and an event per slot
  // that marks its copy done
  static constexpr int kRingSlots = 4;
  char* ring_host = nullptr;
  cudaEvent_t ring_ev[kRingSlots] = {};
  int ring_slot = 0;
  cudaGraphExec_t fgraph = nullptr;
  int fgraph_k = 0, fgraph_cur = -1, fgraph_blk = 0, fgraph_wy = 0, fgraph_kind = -1;
  // asynchronous outputs: a copy stream and a ring of slots; ticket k uses
  // slot k % kOutSlots.  Gauge indices stay on the device between calls.
  cudaStream_t cpy = nullptr;
  OutSlot outs[kOutSlots];
  int64_t out_next = 0;
  int32_t* g_ij = nullptr;
  int g_n = 0, g_cap = 0;
  std::vector<int32_t> g_host;
  // the largest Courant number above 1 that cliffs_gpu_status has cleared
  double courant_seen = 0;
  bool prof = false;
  std::vector<ProfPair> prof_pending;
  double prof_ms[2] = {0, 0};
  int64_t prof_n[2] = {0, 0};
};

namespace {

template <typename T>
int dalloc(T** p, size_t n) {
  if (n == 0) n = 1;
  if (cudaMalloc((void**)p, n * sizeof(T)) != cudaSuccess) return CLIFFS_ERR_NOMEM;
  return CLIFFS_OK;
}

// Reserves n elements of T at the next 256-byte boundary of an arena at
// offset `off`; with base == nullptr it only advances the offset (the sizing
// pass).
template <typename T>
void carve(char* base, size_t& off, T** p, size_t n) {
  off = (off + 255) & ~(size_t)255;
  if (base) *p = reinterpret_cast<T*>(base + off);
  off += (n ? n : 1) * sizeof(T);
}

// dep64 is the caller's FP64 depth.  The device keeps FP32 depths, which a
// deformed bottom need not hit exactly; the surface state is taken against
// the FP64 depth so that the elevation eta = H - dep stays exact and the
// depth's rounding (a relative ~3e-8) goes into the total depth instead.
__global__ void k_init_state(int nx, int ny, int pitch, const double* __restrict__ src,
                             int src_is_celerity, const double* __restrict__ xv,
                             const double* __restrict__ yvv, const float* __restrict__ dep,
                             const double* __restrict__ dep64, float* srf, float* xu, float* yv,
                             double ground, double g) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y;
  if (i >= pitch || j >= ny) return;
  const size_t q = (size_t)j * pitch + i;
  if (i >= nx) {
    srf[q] = 0.f;
    xu[q] = 0.f;
    yv[q] = 0.f;
    return;
  }
  const size_t s = (size_t)j * nx + i;
  const bool land = dep[q] < 0.f;  // the same land test as the sweeps
  double H;
  if (src_is_celerity) {
    const double c = src[s];
    H = c * fabs(c) / g;  // signed total depth keeps the sign of the celerity
  } else {
    // celerity transform of cliffs_main.f:218-227 expressed on H
    H = src[s] <= ground ? 0.0 : src[s];
  }
  srf[q] = (float)(land ? H : H - dep64[s]);  // surface state: H on land, eta at sea
  xu[q] = xv ? (float)xv[s] : 0.f;
  yv[q] = yvv ? (float)yvv[s] : 0.f;
}

// FP32 device depth (pitched, zero padding) from the FP64 depth.
__global__ void k_dep_from64(int nx, int ny, int pitch, const double* __restrict__ dep64, float* dep) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y;
  if (i >= pitch || j >= ny) return;
  dep[(size_t)j * pitch + i] = i < nx ? (float)dep64[(size_t)j * nx + i] : 0.f;
}

__global__ void k_reset_max(int nx, int ny, int pitch, const float* __restrict__ dep, float* hmax,
                            float* velmax) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y;
  if (i >= pitch || j >= ny) return;
  const size_t q = (size_t)j * pitch + i;
  hmax[q] = i < nx ? -dep[q] : 0.f;  // hmax = 0 in celerity form
  velmax[q] = 0.f;
}

__global__ void k_download(int nx, int ny, int pitch, const float* __restrict__ dep,
                           const double* __restrict__ dep64, const float* __restrict__ srf,
                           const float* __restrict__ xu, const float* __restrict__ yv, double* cel,
                           double* xo, double* yo, double g) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y;
  if (i >= nx || j >= ny) return;
  const size_t q = (size_t)j * pitch + i, s = (size_t)j * nx + i;
  // the inverse of k_init_state: eta is exact against the FP64 depth
  const double H = dep[q] < 0.f ? (double)srf[q] : dep64[s] + (double)srf[q];
  if (cel) cel[s] = H < 0 ? -sqrt(-g * H) : sqrt(g * H);
  if (xo) xo[s] = xu[q];
  if (yo) yo[s] = yv[q];
}

__global__ void k_max_raw(int nx, int ny, int pitch, const float* __restrict__ dep,
                          const float* __restrict__ hmax, const float* __restrict__ velmax,
                          double* hout, double* vout, double g) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y;
  if (i >= nx || j >= ny) return;
  const size_t q = (size_t)j * pitch + i, s = (size_t)j * nx + i;
  const double H = (double)dep[q] + (double)hmax[q];
  if (hout) hout[s] = H < 0 ? -sqrt(-g * H) : sqrt(g * H);
  if (vout) vout[s] = velmax[q];
}

// output_maxwave.f:14-27
__global__ void k_maxwave_out(int nx, int ny, int pitch, const float* __restrict__ dep,
                              const float* __restrict__ hmax, const float* __restrict__ velmax,
                              float ground, float* me, float* mv) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y;
  if (i >= nx || j >= ny) return;
  const size_t q = (size_t)j * pitch + i, s = (size_t)j * nx + i;
  const float hm = hmax[q];
  if (dep[q] + hm > ground) {
    me[s] = hm;
    mv[s] = sqrtf(velmax[q]);
  } else {
    me[s] = kNan4;
    mv[s] = kNan4;
  }
}

// output_sea_state.f:18-33
__global__ void k_sea_state(int nxs, int nys, int pitch, int lonsub, int latsub,
                            const float* __restrict__ dep, const float* __restrict__ srf,
                            const float* __restrict__ xu, const float* __restrict__ yv,
                            float ground, float* h, float* u, float* v) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y;
  if (i >= nxs || j >= nys) return;
  const size_t q = (size_t)(latsub * j) * pitch + (size_t)(lonsub * i);
  const size_t s = (size_t)j * nxs + i;
  if (depth_of(srf[q], dep[q]) > ground) {
    h[s] = eta_of(srf[q], dep[q]);
    u[s] = xu[q];
    v[s] = yv[q];
  } else {
    h[s] = kNan4;
    u[s] = kNan4;
    v[s] = kNan4;
  }
}

// output_gages.f:18-29
__global__ void k_gauges(int n, const int32_t* __restrict__ I, const int32_t* __restrict__ J,
                         int pitch, const float* __restrict__ dep, const float* __restrict__ srf,
                         const float* __restrict__ xu, const float* __restrict__ yv, float ground,
                         double* out) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const size_t q = (size_t)(J[k] - 1) * pitch + (size_t)(I[k] - 1);
  const float H = depth_of(srf[q], dep[q]);
  out[k] = H > ground ? (double)eta_of(srf[q], dep[q]) : (double)kNan4;
  out[n + k] = xu[q];
  out[2 * n + k] = yv[q];
}

// Runup measures: per-block partials of (max runup, its index, wetted land
// count, wet count) into scratch, finished on the host.
__global__ void k_runup(int nx, int ny, int pitch, const float* __restrict__ dep,
                        const float* __restrict__ srf, const float* __restrict__ hmax,
                        float ground, double* part) {
  __shared__ double s_best[256];
  __shared__ long long s_idx[256], s_land[256], s_wet[256];
  const int t = threadIdx.x;
  double best = -1.0;
  long long bidx = -1, nland = 0, nwet = 0;
  const long long total = (long long)nx * ny;
  for (long long c = (long long)blockIdx.x * blockDim.x + t; c < total;
       c += (long long)gridDim.x * blockDim.x) {
    const int j = (int)(c / nx), i = (int)(c - (long long)j * nx);
    const size_t q = (size_t)j * pitch + i;
    const float d = dep[q];
    if (depth_of(srf[q], d) > ground) ++nwet;
    if (d < 0.f && d + hmax[q] > ground) {
      ++nland;
      if (-d > best) {
        best = -d;
        bidx = c;
      }
    }
  }
  s_best[t] = best;
  s_idx[t] = bidx;
  s_land[t] = nland;
  s_wet[t] = nwet;
  __syncthreads();
  for (int w = blockDim.x >> 1; w > 0; w >>= 1) {
    if (t < w) {
      if (s_best[t + w] > s_best[t] ||
          (s_best[t + w] == s_best[t] && s_idx[t + w] >= 0 && (s_idx[t] < 0 || s_idx[t + w] < s_idx[t]))) {
        s_best[t] = s_best[t + w];
        s_idx[t] = s_idx[t + w];
      }
      s_land[t] += s_land[t + w];
      s_wet[t] += s_wet[t + w];
    }
    __syncthreads();
  }
  if (t == 0) {
    part[4 * blockIdx.x + 0] = s_best[0];
    part[4 * blockIdx.x + 1] = (double)s_idx[0];
    part[4 * blockIdx.x + 2] = (double)s_land[0];
    part[4 * blockIdx.x + 3] = (double)s_wet[0];
  }
}

// Arrival test of feed_children_grid.f:26-46 over parent columns ii1..ii2 and
// rows kk1..kk2 (1-based).
__global__ void k_arrival(int ii1, int ii2, int kk1, int kk2, int pitch,
                          const float* __restrict__ dep, const float* __restrict__ srf,
                          const float* __restrict__ xu, const float* __restrict__ yv,
                          double hmin, double cuke, double g, int* flag, bool sticky) {
  if (sticky && *(volatile int*)flag) return;  // arrived at an earlier call
  const int ni = ii2 - ii1 + 1, nk = kk2 - kk1 + 1;
  const long long total = (long long)ni * nk;
  const double tenth = (double)0.1f;
  bool hit = false;
  for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < total && !hit;
       c += (long long)gridDim.x * blockDim.x) {
    const int k = kk1 + (int)(c / ni), i = ii1 + (int)(c % ni);
    const size_t q = (size_t)(k - 1) * pitch + (size_t)(i - 1);
    const double d = dep[q];
    if (d > hmin) {
      const double H = depth_of((double)srf[q], d);
      const double c2g = fabs(H);  // cel**2/grav
      if (fabs(c2g - d) > tenth * cuke) hit = true;
      const double cel = H < 0 ? -sqrt(-g * H) : sqrt(g * H);
      if ((fabs((double)xu[q]) + fabs((double)yv[q])) * cel > cuke) hit = true;
    }
  }
  if (hit) atomicOr(flag, 1);
}

// Edge records of feed_children_grid.f:47-177; one thread per child edge node.
__device__ __forceinline__ void feed_clm(int i, int k, int pitch, const float* dep,
                                         const float* srf, const float* xu, const float* yv,
                                         double cc, double hmin, double g, double out[3]) {
  const size_t q = (size_t)(k - 1) * pitch + (size_t)(i - 1);
  const double d = dep[q];
  if (d > hmin) {
    const double H = depth_of((double)srf[q], d);
    out[0] = cc * (double)xu[q];
    out[1] = cc * (double)yv[q];
    out[2] = cc * (fabs(H) - d);
    (void)g;
  } else {
    out[0] = out[1] = out[2] = 0.0;
  }
}

__global__ void k_feed_child(int mm, int nn, int W_nx, int E_nx, int S_ny, int N_ny, double W_cx,
                             double E_cx, double S_cy, double N_cy, const int32_t* __restrict__ WE_ny,
                             const double* __restrict__ WE_cy, const int32_t* __restrict__ SN_nx,
                             const double* __restrict__ SN_cx, int pitch, const float* __restrict__ dep,
                             const float* __restrict__ srf, const float* __restrict__ xu,
                             const float* __restrict__ yv, double hmin, double g, double* w_out,
                             double* e_out, double* s_out, double* n_out, const int* gate, int* gate_out) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (gate) {  // the asynchronous feed: no record before the wave reaches the child
    const int open = *gate;
    if (t == 0) *gate_out = open;  // the flag as this record saw it, for the host
    if (!open) return;
  }
  if (t < 2 * nn) {  // west / east: parent columns (ii, ii+1), rows kk, kk+1
    const int side = t / nn, i = t % nn;
    const int ii = side == 0 ? W_nx : E_nx;
    const double cc = side == 0 ? W_cx : E_cx;
    const int kk = WE_ny[i];
    const double w = WE_cy[i];
    double a0[3], a1[3], b0[3], b1[3];
    feed_clm(ii, kk, pitch, dep, srf, xu, yv, cc, hmin, g, a0);
    feed_clm(ii + 1, kk, pitch, dep, srf, xu, yv, 1 - cc, hmin, g, a1);
    feed_clm(ii, kk + 1, pitch, dep, srf, xu, yv, cc, hmin, g, b0);
    feed_clm(ii + 1, kk + 1, pitch, dep, srf, xu, yv, 1 - cc, hmin, g, b1);
    double* o = side == 0 ? w_out : e_out;
    for (int c = 0; c < 3; ++c) o[i + (size_t)c * nn] = (a0[c] + a1[c]) * w + (b0[c] + b1[c]) * (1 - w);
  } else if (t < 2 * nn + 2 * mm) {  // south / north: parent rows (kk, kk+1)
    const int u = t - 2 * nn;
    const int side = u / mm, i = u % mm;
    const int kk = side == 0 ? S_ny : N_ny;
    const double cc = side == 0 ? S_cy : N_cy;
    const int ii = SN_nx[i];
    const double w = SN_cx[i];
    double a0[3], a1[3], b0[3], b1[3];
    feed_clm(ii, kk, pitch, dep, srf, xu, yv, cc, hmin, g, a0);
    feed_clm(ii, kk + 1, pitch, dep, srf, xu, yv, 1 - cc, hmin, g, a1);
    feed_clm(ii + 1, kk, pitch, dep, srf, xu, yv, cc, hmin, g, b0);
    feed_clm(ii + 1, kk + 1, pitch, dep, srf, xu, yv, 1 - cc, hmin, g, b1);
    double* o = side == 0 ? s_out : n_out;
    for (int c = 0; c < 3; ++c) o[i + (size_t)c * mm] = (a0[c] + a1[c]) * w + (b0[c] + b1[c]) * (1 - w);
  }
}

int check_device(int* dev) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) return CLIFFS_ERR_DEVICE;
  if (cudaGetDevice(dev) != cudaSuccess) return CLIFFS_ERR_DEVICE;
  cudaDeviceProp pr;
  if (cudaGetDeviceProperties(&pr, *dev) != cudaSuccess) return CLIFFS_ERR_DEVICE;
  if (pr.major < 10) return CLIFFS_ERR_DEVICE;
  return CLIFFS_OK;
}

Phys<float> phys(const cliffs_ctx* c) {
  Phys<float> p;
  p.g = (float)kGrav;
  p.ginv = (float)(1.0 / kGrav);
  p.ground = (float)c->ground;
  p.celmin = (float)c->celmin;
  p.dt = (float)c->dt;
  p.idt = (float)(1.0 / c->dt);
  p.gcrough = (float)(kGrav * c->crough);
  p.sqr2 = (float)kSqr2;
  return p;
}

dim3 grid2(int nx, int ny, int bx = 128) { return dim3((nx + bx - 1) / bx, ny); }

constexpr int kGeneralBlocks = 304;

// Launch one sweep: the fast kernel, then the general kernel over the cells it
// listed.  fuse_max: update hmax/velmax on the way out.
// ---- analytic sources (cliffs_gpu_add_source) --------------------------------

struct SourceParams {
  double x0, y0, ax, ay, ca, sa, amp, dipole;
};

// Uplift of an elliptical Gaussian with its first axis rotated by angle from
// +x, minus a trough of relative depth `dipole` two half-widths along the
// second axis.
__device__ __forceinline__ double source_at(const SourceParams& S, double x, double y) {
  const double dx = x - S.x0, dy = y - S.y0;
  const double xi = S.ca * dx + S.sa * dy, et = -S.sa * dx + S.ca * dy;
  const double a = xi / S.ax, b = et / S.ay, b2 = (et + 2.0 * S.ay) / S.ay;
  return S.amp * (exp(-(a * a + b * b)) - S.dipole * exp(-(a * a + b2 * b2)));
}

__global__ void k_source(int nx, int ny, int pitch, const double* __restrict__ x, const double* __restrict__ y,
                         SourceParams S, float* q) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y;
  if (i >= pitch || j >= ny) return;
  q[(size_t)j * pitch + i] = i < nx ? (float)source_at(S, x[i], y[j]) : 0.f;
}

// apply_initial_conditions.f:7-70 on the device: the bilinear value of a
// lattice q (nxq x nyq, x fastest) at every grid node.  The host has placed
// the grid's columns and rows in the lattice (pinpoint): ii/jj 1-based, -1
// for a node outside it, xc/yc the weights of the lower lattice node.  A
// lattice one node wide along an axis interpolates along the other only.
__global__ void k_lattice(int nx, int ny, int pitch, const int32_t* __restrict__ ii, const double* __restrict__ xc,
                          const int32_t* __restrict__ jj, const double* __restrict__ yc, int nxq, int nyq,
                          const double* __restrict__ q, float* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y;
  if (i >= pitch || j >= ny) return;
  double v = 0.0;
  if (i < nx) {
    auto Q = [&](int a, int b) { return q[(size_t)(b - 1) * nxq + (a - 1)]; };
    if (nxq > 2 && nyq > 2) {
      const int a = ii[i], b = jj[j];
      if (a > 0 && b > 0) {
        const double x = xc[i], y = yc[j];
        v = (Q(a, b) * x + Q(a + 1, b) * (1 - x)) * y + (Q(a, b + 1) * x + Q(a + 1, b + 1) * (1 - x)) * (1 - y);
      }
    } else if (nyq == 1 && nxq > 2) {
      const int a = ii[i];
      if (a > 0) v = Q(a, 1) * xc[i] + Q(a + 1, 1) * (1 - xc[i]);
    } else if (nxq == 1 && nyq > 2) {
      const int b = jj[j];
      if (b > 0) v = Q(1, b) * yc[j] + Q(1, b + 1) * (1 - yc[j]);
    }
  }
  out[(size_t)j * pitch + i] = (float)v;
}

// A field q (pitched FP32) added to the velocity component u (or v).
__global__ void k_add_field(int nx, int ny, int pitch, float* f, const float* __restrict__ q) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y;
  if (i >= nx || j >= ny) return;
  const size_t k = (size_t)j * pitch + i;
  f[k] += q[k];
}

// The surface rises by (w_now - w_prev) q where water stands; a dry cell takes
// the water column dep + w_now q once that exceeds ground, as the initial
// surface deformation of cliffs_main.f:209-213 does before the celerity
// transform.
__global__ void k_add_surface(int nx, int ny, int pitch, const float* __restrict__ dep, float* srf,
                              const float* __restrict__ q, float w_now, float w_prev, float ground) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y;
  if (i >= nx || j >= ny) return;
  const size_t k = (size_t)j * pitch + i;
  const float d = dep[k], s = srf[k], qq = q[k];
  if (depth_of(s, d) > ground) {
    srf[k] = s + (w_now - w_prev) * qq;  // eta and H move together
  } else {
    const float Hd = d + w_now * qq;
    if (Hd > ground) srf[k] = state_from_depth(Hd, d);
  }
}

// The bottom rises by q (pitched FP32) under a standing water column
// (cliffs_main.f:205-208).  The FP64 depth moves and the FP32 depth becomes
// its rounding.  eta rises where it is sea before and after, the depth stays
// where it is land before and after, and a cell changing sides converts
// through its total depth.
__global__ void k_move_bottom64(int nx, int ny, int pitch, const float* __restrict__ q, double* dep64,
                                float* dep, float* srf) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y;
  if (i >= nx || j >= ny) return;
  const size_t k = (size_t)j * pitch + i, s = (size_t)j * nx + i;
  const double d = dep64[s] - (double)q[k];
  dep64[s] = d;
  const float d0 = dep[k], d1 = (float)d, v = srf[k];
  dep[k] = d1;
  if (d0 >= 0.f && d1 >= 0.f)
    srf[k] = v + (d0 - d1);
  else if (!(d0 < 0.f && d1 < 0.f))
    srf[k] = state_from_depth(depth_of(v, d0), d1);
}

// The arguments of one sweep reading state copy s and writing 1 - s.
SweepArgs sweep_args(const cliffs_ctx* c, int iu, bool fuse_max, int s) {
  SweepArgs A{};
  const int o = 1 - s;
  A.pitch = c->pitch;
  A.dep = c->dep;
  A.srf = c->srf[s];
  A.xu = c->xu[s];
  A.yv = c->yv[s];
  A.srf_o = c->srf[o];
  A.xu_o = c->xu[o];
  A.yv_o = c->yv[o];
  A.hmax = fuse_max ? c->hmax : nullptr;
  A.velmax = fuse_max ? c->velmax : nullptr;
  A.ph = phys(c);
  A.status = c->status;
  A.list = c->list;
  A.count = c->cnt + (c->sweeps & 1u);
  A.count_next = c->cnt + ((c->sweeps + 1u) & 1u);
  A.edges = nullptr;
  if (iu == 1) {
    A.n = c->nx;
    A.nlines = c->ny;
    A.lo = c->jj1;
    A.hi = c->jj2;
    A.geo = c->geo_x;
    A.geo_uniform = c->geo_uni_x;
    A.geo0 = c->geo0_x;
    A.scl = nullptr;
    A.lscale = c->lscale;
    A.inv_dx1 = c->inv_dx1_x;
    A.inv_dxn1 = c->inv_dxn1_x;
  } else {
    A.n = c->ny;
    A.nlines = c->nx;
    A.lo = c->ii1;
    A.hi = c->ii2;
    A.geo = c->geo_y;
    A.geo_uniform = c->geo_uni_y;
    A.geo0 = c->geo0_y;
    A.scl = c->scl_y;
    A.lscale = nullptr;
    A.inv_dx1 = c->inv_dx1_y;
    A.inv_dxn1 = c->inv_dxn1_y;
  }
  return A;
}

// One fast-kernel sweep on the context's stream, a programmatic dependent of
// the previous launch when c->pdl is set.
template <int DIR, bool MAXOUT>
cudaError_t launch_fast(cliffs_ctx* c, dim3 grid, unsigned block, const SweepArgs& A) {
  const bool flat = A.geo_uniform && A.scl == nullptr;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = dim3(block);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = c->stream;
  cfg.attrs = at;
  cfg.numAttrs = c->pdl ? 1 : 0;
  return flat ? cudaLaunchKernelEx(&cfg, fast_kernel<DIR, true, MAXOUT, true>, A)
              : cudaLaunchKernelEx(&cfg, fast_kernel<DIR, true, MAXOUT, false>, A);
}

// Max-wave handling of one sweep: none, the update with its outputs (the last
// sweep of a step in one dimension, or with the staged kernels), or the fold
// of its input (the x-sweep of a two-dimensional step, tiled kernels).
enum { MAXM_NONE = 0, MAXM_OUT = 1, MAXM_IN = 2 };

int launch_sweep(cliffs_ctx* c, int iu, int maxm, const double* fA, const double* fB,
                 int flen, int irec, double cc, const float* pre = nullptr) {
  SweepArgs A = sweep_args(c, iu, maxm == MAXM_OUT, c->cur);
  if (maxm == MAXM_IN && iu == 1) {
    A.hmax_in = c->hmax;
    A.velmax_in = c->velmax;
  }
  const int o = 1 - c->cur;
  if (pre) {  // this step's edge table, already in the ring
    A.edges = pre;
  } else if (fA || fB) {
    float* eb = iu == 1 ? c->edge_x : c->edge_y;
    const int nl = iu == 1 ? c->ny : c->nx;
    ++c->launches;
    edges_kernel<<<(nl + 127) / 128, 128, 0, c->stream>>>(nl, flen, fA, fB, irec, cc, iu == 1 ? 0 : 1,
                                                          iu == 1 ? 1 : 0, eb);
    CK(cudaGetLastError());
    A.edges = eb;
  }
  ProfPair pp{};
  if (c->prof) {
    CK(cudaEventCreate(&pp.a));
    CK(cudaEventCreate(&pp.b));
    pp.dir = iu - 1;
    CK(cudaEventRecord(pp.a, c->stream));
  }
  const bool staged = c->sweep_kind == CLIFFS_SWEEP_STAGED && c->staged_ok;
  if (staged) {
    const StageCtl S{c->stage_ns, 0u};
    ++c->launches;
    if (iu == 1) {
      const int tiles = (A.n + kXTile - 1) / kXTile * A.nlines;
      staged_x<<<std::min(tiles, c->grid_sx), kStagedThreads, 0, c->stream>>>(A, S);
    } else {
      const int tiles = (A.n + kYRows - 1) / kYRows * ((A.nlines + 31) / 32);
      const YMaps M{c->m_dep, c->m_srf[c->cur], c->m_xu[c->cur], c->m_yv[c->cur], c->m_hmax, c->m_velmax};
      staged_y<<<std::min(tiles, c->grid_sy), kStagedThreads, 0, c->stream>>>(A, M, S);
    }
  } else if (iu == 1) {
    const int cells = c->blk_x * kCellsPerThread;
    const dim3 grid((A.n + cells - 1) / cells, A.nlines);
    ++c->launches;
    if (maxm == MAXM_OUT)
      CK((launch_fast<0, true>(c, grid, (unsigned)c->blk_x, A)));
    else
      CK((launch_fast<0, false>(c, grid, (unsigned)c->blk_x, A)));
  } else if (c->sweep_kind == CLIFFS_SWEEP_TILED && c->ytile_ok && maxm != MAXM_OUT && c->warps_y == 4) {
    // the y-sweep of a two-dimensional step: tiles staged by the copy engine
    const dim3 grid((A.nlines + 31) / 32, (A.n + kYRows - 1) / kYRows);  // (column groups, bands)
    const int s = c->cur;
    const YTileMaps M{c->m_dep, c->m_srf[s], c->m_xu[s], c->m_yv[s], c->m_srf16[1 - s], c->m_xu16[1 - s],
                      c->m_yv16[1 - s]};
    const StageCtl S{c->stage_ns, 0u};
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = dim3(kStagedThreads);
    cfg.stream = c->stream;
    cfg.attrs = at;
    cfg.numAttrs = c->pdl ? 1 : 0;
    ++c->launches;
    if (A.geo_uniform && A.scl == nullptr)
      CK(cudaLaunchKernelEx(&cfg, tile_y_kernel<true>, A, M, S));
    else
      CK(cudaLaunchKernelEx(&cfg, tile_y_kernel<false>, A, M, S));
  } else {
    const int rows = c->warps_y * kCellsPerThread;
    const dim3 grid((A.nlines + 31) / 32, (A.n + rows - 1) / rows);  // (column groups, bands)
    ++c->launches;
    if (maxm == MAXM_OUT)
      CK((launch_fast<1, true>(c, grid, (unsigned)(32 * c->warps_y), A)));
    else
      CK((launch_fast<1, false>(c, grid, (unsigned)(32 * c->warps_y), A)));
  }
  CK(cudaGetLastError());
  if (c->prof) {
    CK(cudaEventRecord(pp.b, c->stream));
    c->prof_pending.push_back(pp);
  }
  c->cur = o;
  c->sweeps += 1u;
  return CLIFFS_OK;
}

__global__ void k_maxwave_update(int nx, int ny, int pitch, const float* __restrict__ dep,
                                 const float* __restrict__ srf, const float* __restrict__ xu,
                                 const float* __restrict__ yv, float* hmax, float* velmax) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y;
  if (i >= nx || j >= ny) return;
  const size_t q = (size_t)j * pitch + i;
  const float eta = eta_of(srf[q], dep[q]);
  if (eta > hmax[q]) hmax[q] = eta;
  const float s = xu[q] * xu[q] + yv[q] * yv[q];
  if (s > velmax[q]) velmax[q] = s;
}

// The end state of the latest step into the max-wave fields, if the next
// x-sweep has not folded it in yet: before hmax/velmax are read or the state
// is changed outside a step.
int max_sync(cliffs_ctx* c) {
  if (!c->max_pending) return CLIFFS_OK;
  ++c->launches;
  k_maxwave_update<<<grid2(c->nx, c->ny), 128, 0, c->stream>>>(c->nx, c->ny, c->pitch, c->dep, c->srf[c->cur],
                                                              c->xu[c->cur], c->yv[c->cur], c->hmax, c->velmax);
  CK(cudaGetLastError());
  c->max_pending = false;
  return CLIFFS_OK;
}

// The max-wave handling of the two sweeps of a step (see MAXM_*).
void step_modes(const cliffs_ctx* c, int* mx, int* my) {
  if (c->sweep_kind == CLIFFS_SWEEP_STAGED && c->staged_ok) {
    *mx = c->yrun ? MAXM_NONE : MAXM_OUT;
    *my = MAXM_OUT;
  } else if (c->xrun && c->yrun) {
    *mx = c->max_fresh ? MAXM_NONE : MAXM_IN;
    *my = MAXM_NONE;
  } else {
    *mx = MAXM_OUT;
    *my = MAXM_OUT;
  }
}

// After a step: with the fold, its end state is pending.
void step_done(cliffs_ctx* c) {
  int mx, my;
  step_modes(c, &mx, &my);
  c->max_pending = my == MAXM_NONE && c->xrun && c->yrun;
  c->max_fresh = false;
}

int flush_profile(cliffs_ctx* c) {
  if (c->prof_pending.empty()) return CLIFFS_OK;
  CK(cudaStreamSynchronize(c->stream));
  for (auto& p : c->prof_pending) {
    float ms = 0;
    CK(cudaEventElapsedTime(&ms, p.a, p.b));
    c->prof_ms[p.dir] += ms;
    c->prof_n[p.dir] += 1;
    cudaEventDestroy(p.a);
    cudaEventDestroy(p.b);
  }
  c->prof_pending.clear();
  return CLIFFS_OK;
}

}  // namespace

extern "C" {

const char* cliffs_gpu_strerror(int code) {
  switch (code) {
    case CLIFFS_OK: return "ok";
    case CLIFFS_FEED_ENDED: return "boundary forcing ended (freeze)";
    case CLIFFS_WARN_CFL: return "a sweep read a state with a Courant number above 1";
    case CLIFFS_ERR_ARG: return "invalid argument";
    case CLIFFS_ERR_CUDA: return "CUDA runtime error";
    case CLIFFS_ERR_NAN: return "non-finite value in the state";
    case CLIFFS_ERR_NOMEM: return "device allocation failed";
    case CLIFFS_ERR_STATE: return "call out of order";
    case CLIFFS_ERR_DEVICE: return "no usable sm_103 device";
    case CLIFFS_ERR_TIMEOUT: return "a device-side wait ran out";
    default: return "unknown status";
  }
}

int cliffs_gpu_metrics(int32_t nx, int32_t ny, int32_t cartesian, const double* xcrd,
                       const double* ycrd, double* dx, double* row_scale, double* dy, double* zeta) {
  if (nx < 1 || ny < 1 || !xcrd || !ycrd) return CLIFFS_ERR_ARG;
  const double beta = kPi * kEarthR / 180.;  // MasterGrid.f:85
  if (nx > 2) {
    if (dx)
      for (int i = 0; i < nx - 1; ++i)
        dx[i] = cartesian ? xcrd[i + 1] - xcrd[i] : beta * (xcrd[i + 1] - xcrd[i]);
    if (row_scale)
      for (int j = 0; j < ny; ++j) row_scale[j] = cartesian ? 1.0 : cos(kPi / 180. * ycrd[j]);
  }
  if (ny > 2) {
    if (dy)
      for (int j = 0; j < ny - 1; ++j)
        dy[j] = cartesian ? ycrd[j + 1] - ycrd[j] : beta * (ycrd[j + 1] - ycrd[j]);
    if (zeta)
      for (int j = 0; j < ny; ++j)
        zeta[j] = cartesian ? 0.0 : (0.125 / kEarthR) * tan(kPi / 180. * ycrd[j]);
  }
  return CLIFFS_OK;
}

int cliffs_gpu_create(const cliffs_grid_desc* d, cliffs_ctx** out) {
  if (!d || !out || !d->dep || d->nx < 1 || d->ny < 1) return CLIFFS_ERR_ARG;
  if (d->nx <= 2 && d->ny <= 2) return CLIFFS_ERR_ARG;
  if (d->nx > 2 && !d->dx) return CLIFFS_ERR_ARG;
  if (d->ny > 2 && !d->dy) return CLIFFS_ERR_ARG;
  if (!(d->dt > 0) || !(d->ground > 0) || d->crough < 0) return CLIFFS_ERR_ARG;
  // launch limits: the x-sweep's grid has a block row per grid row, the
  // y-sweep's one per band of 16 rows (65535 block rows at most)
  if (d->nx > 2 && d->ny > 65535) return CLIFFS_ERR_ARG;
  if (d->ny > 2 && (d->ny + 15) / 16 > 65535) return CLIFFS_ERR_ARG;
  int dev = 0;
  int r = check_device(&dev);
  if (r) return r;
  cliffs_ctx* c = new cliffs_ctx();
  c->dev = dev;
  if (const char* e = getenv("CLIFFS_PDL")) c->pdl = std::strcmp(e, "0") != 0;
  c->nx = d->nx;
  c->ny = d->ny;
  c->pitch = (d->nx + 31) / 32 * 32;
  c->ground = d->ground;
  c->crough = d->crough;
  c->dt = d->dt;
  c->celmin = sqrt(kGrav * d->ground);  // cliffs_main.f:227
  // 1-D / 2-D detection (cliffs_main.f:140-164)
  c->xrun = d->nx > 2;
  c->yrun = d->ny > 2;
  c->ii1 = c->xrun ? 2 : 1;
  c->ii2 = c->xrun ? d->nx - 1 : 1;
  c->jj1 = c->yrun ? 2 : 1;
  c->jj2 = c->yrun ? d->ny - 1 : 1;
  const size_t cells = (size_t)c->pitch * c->ny;
  auto fail = [&](int code) {
    cliffs_gpu_destroy(c);
    return code;
  };
  if (cudaStreamCreateWithFlags(&c->own, cudaStreamNonBlocking) != cudaSuccess) return fail(CLIFFS_ERR_CUDA);
  c->stream = c->own;
  const size_t n64 = (size_t)c->nx * c->ny;
  auto layout = [&](char* base) {
    size_t off = 0;
    carve(base, off, &c->dep, cells);
    for (int k = 0; k < 2; ++k) {
      carve(base, off, &c->srf[k], cells);
      carve(base, off, &c->xu[k], cells);
      carve(base, off, &c->yv[k], cells);
    }
    carve(base, off, &c->hmax, cells);
    carve(base, off, &c->velmax, cells);
    carve(base, off, &c->geo_x, (size_t)c->nx);
    carve(base, off, &c->geo_y, (size_t)c->ny);
    carve(base, off, &c->scl_y, (size_t)c->ny);
    carve(base, off, &c->lscale, (size_t)c->ny);
    carve(base, off, &c->status, 2);
    carve(base, off, &c->d_flag, 1);
    carve(base, off, &c->list, n64);
    carve(base, off, &c->edge_x, (size_t)c->ny * 6);
    carve(base, off, &c->edge_y, (size_t)c->nx * 6);
    carve(base, off, &c->cnt, 2);
    carve(base, off, &c->dep64, n64);
    carve(base, off, &c->xfer, 3 * n64);
    return off;
  };
  if (dalloc(&c->arena, layout(nullptr))) return fail(CLIFFS_ERR_NOMEM);
  layout(c->arena);
  // bathymetry: the FP64 depth as passed, and its rounding in padded rows;
  // the host builds the geometry meanwhile, and one synchronisation at the
  // end covers both
  if (cudaMemcpyAsync(c->dep64, d->dep, (size_t)c->nx * c->ny * sizeof(double), cudaMemcpyHostToDevice,
                      c->stream) != cudaSuccess)
    return fail(CLIFFS_ERR_CUDA);
  ++c->launches;
  k_dep_from64<<<grid2(c->pitch, c->ny), 128, 0, c->stream>>>(c->nx, c->ny, c->pitch, c->dep64, c->dep);
  if (cudaGetLastError() != cudaSuccess) return fail(CLIFFS_ERR_CUDA);
  // geometry tables
  auto build_geo = [&](int n, const double* s, std::vector<float4>& geo, float& i1, float& in1) {
    geo.assign((size_t)n, make_float4(0, 0, 0, 0));
    for (int m = 2; m <= n - 1; ++m) {
      const double fm = s[m - 2], fp = s[m - 1];
      geo[m - 1] = make_float4((float)(1.0 / fm), (float)(1.0 / fp), (float)(d->dt / (fm + fp)), (float)(fp - fm));
    }
    i1 = (float)(1.0 / s[0]);
    in1 = (float)(1.0 / s[n - 2]);
  };
  std::vector<float4> gx, gy;
  if (c->xrun) build_geo(c->nx, d->dx, gx, c->inv_dx1_x, c->inv_dxn1_x);
  else gx.assign((size_t)c->nx, make_float4(0, 0, 0, 0));
  if (c->yrun) build_geo(c->ny, d->dy, gy, c->inv_dx1_y, c->inv_dxn1_y);
  else gy.assign((size_t)c->ny, make_float4(0, 0, 0, 0));
  // An axis is uniform when every spacing equals the first within 1e-9 of
  // it: a longitude axis in FP64 degrees has spacings that differ in the
  // 12th digit, below what the FP32 geometry keeps except in dx(m)-dx(m-1).
  // A uniform axis takes the geometry of its first spacing everywhere (the
  // table too, so that every kernel variant reads the same values): the
  // table of an exactly uniform axis is unchanged by it.
  auto uniform = [&](int n, const double* sp, std::vector<float4>& g, float4& g0) {
    if (n < 3) return false;
    const double s0 = sp[0];
    for (int k = 1; k <= n - 2; ++k)
      if (std::fabs(sp[k] - s0) > 1e-9 * std::fabs(s0)) return false;
    g0 = make_float4((float)(1.0 / s0), (float)(1.0 / s0), (float)(d->dt / (s0 + s0)), 0.f);
    for (int m = 2; m <= n - 1; ++m) g[m - 1] = g0;
    return true;
  };
  if (c->xrun) c->geo_uni_x = uniform(c->nx, d->dx, gx, c->geo0_x);
  if (c->yrun) c->geo_uni_y = uniform(c->ny, d->dy, gy, c->geo0_y);
  std::vector<float> sy((size_t)c->ny, 0.f);
  bool zeta_nonzero = false;
  if (d->zeta)
    for (int j = 0; j < c->ny; ++j) {
      sy[j] = (float)d->zeta[j];
      zeta_nonzero |= sy[j] != 0.f;
    }
  std::vector<float2> ls((size_t)c->ny, make_float2(1.f, 1.f));
  if (d->row_scale)
    for (int j = 0; j < c->ny; ++j) ls[j] = make_float2((float)d->row_scale[j], (float)(1.0 / d->row_scale[j]));
  {
    // the four tables lie one after another in the arena: one copy of their
    // span, laid out on the host as there
    char* const lo = reinterpret_cast<char*>(c->geo_x);
    char* const hi = reinterpret_cast<char*>(c->lscale + c->ny);
    std::vector<char> span((size_t)(hi - lo), 0);
    auto put = [&](const void* dev, const void* src, size_t bytes) {
      std::memcpy(span.data() + (reinterpret_cast<const char*>(dev) - lo), src, bytes);
    };
    put(c->geo_x, gx.data(), gx.size() * sizeof(float4));
    put(c->geo_y, gy.data(), gy.size() * sizeof(float4));
    put(c->scl_y, sy.data(), sy.size() * sizeof(float));
    put(c->lscale, ls.data(), ls.size() * sizeof(float2));
    if (cudaMemcpyAsync(lo, span.data(), span.size(), cudaMemcpyHostToDevice, c->stream) != cudaSuccess ||
        cudaMemsetAsync(c->status, 0, 2 * sizeof(unsigned), c->stream) != cudaSuccess ||
        cudaMemsetAsync(c->cnt, 0, 2 * sizeof(uint32_t), c->stream) != cudaSuccess ||
        cudaStreamSynchronize(c->stream) != cudaSuccess)
      return fail(CLIFFS_ERR_CUDA);
  }
  if (!d->row_scale) c->lscale = nullptr;  // (its arena slot stays unused)
  if (!zeta_nonzero) c->scl_y = nullptr;
  // the staged sweep kernels: tensor maps of the y-sweep's fields and the
  // resident grid of each kernel; without them the context keeps fast_kernel
  {
    // the device's SM count and the staged kernels' resident blocks, asked
    // once per device and process
    static std::mutex occ_mu;
    static int occ[64][3] = {};
    int nsm = 0, bx = 0, by = 0;
    {
      std::lock_guard<std::mutex> lk(occ_mu);
      const bool cached = dev < 64 && occ[dev][0] > 0;
      if (cached) {
        nsm = occ[dev][0];
        bx = occ[dev][1];
        by = occ[dev][2];
      } else if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess &&
                 cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bx, staged_x, kStagedThreads, 0) == cudaSuccess &&
                 cudaOccupancyMaxActiveBlocksPerMultiprocessor(&by, staged_y, kStagedThreads, 0) == cudaSuccess &&
                 dev < 64 && nsm > 0) {
        occ[dev][0] = nsm;
        occ[dev][1] = bx;
        occ[dev][2] = by;
      }
    }
    bool ok = get_encoder() == CLIFFS_OK && nsm > 0 && bx > 0 && by > 0;
    const int nx = c->nx, ny = c->ny, pp = c->pitch;
    ok = ok && !make_map(&c->m_dep, c->dep, nx, ny, pp, 32, kYWin) && !make_map(&c->m_hmax, c->hmax, nx, ny, pp, 32, kYRows) &&
         !make_map(&c->m_velmax, c->velmax, nx, ny, pp, 32, kYRows);
    for (int k = 0; k < 2 && ok; ++k)
      ok = !make_map(&c->m_srf[k], c->srf[k], nx, ny, pp, 32, kYWin) &&
           !make_map(&c->m_xu[k], c->xu[k], nx, ny, pp, 32, kYWin) &&
           !make_map(&c->m_yv[k], c->yv[k], nx, ny, pp, 32, kYWin);
    c->staged_ok = ok;
    bool yt = ok;
    for (int k = 0; k < 2 && yt; ++k)
      yt = !make_map(&c->m_srf16[k], c->srf[k], nx, ny, pp, 32, kYRows) &&
           !make_map(&c->m_xu16[k], c->xu[k], nx, ny, pp, 32, kYRows) &&
           !make_map(&c->m_yv16[k], c->yv[k], nx, ny, pp, 32, kYRows);
    c->ytile_ok = yt;
    c->grid_sx = nsm * bx;
    c->grid_sy = nsm * by;
  }
  *out = c;
  return CLIFFS_OK;
}

void cliffs_gpu_destroy(cliffs_ctx* c) {
  if (!c) return;
  cudaStreamSynchronize(c->stream);
  flush_profile(c);
  void* ptrs[] = {c->arena, c->fw, c->fe, c->fs, c->fn, c->edge_s[0], c->edge_s[1], c->red,
                  c->rise_q, c->ring_x, c->ring_y, c->ring_irec, c->ring_cc};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  for (auto& n : c->nests) {
    cudaFree(n.WE_ny);
    cudaFree(n.WE_cy);
    cudaFree(n.SN_nx);
    cudaFree(n.SN_cx);
    cudaFree(n.d_arr);
  }
  if (c->cpy) cudaStreamSynchronize(c->cpy);
  for (auto& o : c->outs) {
    if (o.dbuf) cudaFree(o.dbuf);
    if (o.conv) cudaEventDestroy(o.conv);
    if (o.done) cudaEventDestroy(o.done);
  }
  if (c->g_ij) cudaFree(c->g_ij);
  if (c->cpy) cudaStreamDestroy(c->cpy);
  for (auto& pg : c->pgraph)
    if (pg.exec) cudaGraphExecDestroy(pg.exec);
  if (c->fgraph) cudaGraphExecDestroy(c->fgraph);
  if (c->ring_host) cudaFreeHost(c->ring_host);
  for (cudaEvent_t e : c->ring_ev)
    if (e) cudaEventDestroy(e);
  if (c->own) cudaStreamDestroy(c->own);
  delete c;
}

int cliffs_gpu_set_stream(cliffs_ctx* c, void* stream) {
  if (!c) return CLIFFS_ERR_ARG;
  CK(cudaStreamSynchronize(c->stream));
  c->stream = stream ? (cudaStream_t)stream : c->own;
  return CLIFFS_OK;
}

// The device's address of a caller's host array when kernels can read and
// write it in place: pinned memory (cliffs_gpu_host_alloc, cudaHostAlloc,
// cudaHostRegister).  nullptr for pageable memory, which goes through the
// staging area and the copy engines.  On GB300 a kernel moves pinned host
// memory over the host link as fast as the copy engines do (~200 GB/s each
// way), so converting in place saves the staging pass and overlaps the
// conversion with the transfer.
static void* host_mapped(const void* p, int dev) {
  if (!p) return nullptr;
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    (void)cudaGetLastError();
    return nullptr;
  }
  // pinned for this context's device (an allocation made with another device
  // current, and not portable, takes the staging path)
  return a.type == cudaMemoryTypeHost && a.device == dev ? a.devicePointer : nullptr;
}

// The FP64 transfer staging of a context: three nx*ny arrays of doubles.
static int xfer_area(cliffs_ctx* c, double** out) {
  if (!c->xfer && dalloc(&c->xfer, 3 * (size_t)c->nx * c->ny)) return CLIFFS_ERR_NOMEM;
  *out = c->xfer;
  return CLIFFS_OK;
}

static int upload_common(cliffs_ctx* c, const double* src, int is_cel, const double* xv,
                         const double* yv, bool reset_max) {
  if (!c || !src) return CLIFFS_ERR_ARG;
  const size_t n = (size_t)c->nx * c->ny;
  double* x = nullptr;
  RET(xfer_area(c, &x));
  const double *dsrc = x, *dx = xv ? x + n : nullptr, *dy = yv ? x + 2 * n : nullptr;
  int r = CLIFFS_OK;
  const double *ms = (const double*)host_mapped(src, c->dev), *mx = (const double*)host_mapped(xv, c->dev),
               *my = (const double*)host_mapped(yv, c->dev);
  if (ms && (!xv || mx) && (!yv || my)) {  // pinned: k_init_state reads the caller's arrays in place
    dsrc = ms;
    dx = mx;
    dy = my;
  } else {
    if (cudaMemcpyAsync(x, src, n * sizeof(double), cudaMemcpyHostToDevice, c->stream)) r = CLIFFS_ERR_CUDA;
    if (!r && xv && cudaMemcpyAsync(x + n, xv, n * sizeof(double), cudaMemcpyHostToDevice, c->stream))
      r = CLIFFS_ERR_CUDA;
    if (!r && yv && cudaMemcpyAsync(x + 2 * n, yv, n * sizeof(double), cudaMemcpyHostToDevice, c->stream))
      r = CLIFFS_ERR_CUDA;
  }
  if (!r && !reset_max && c->have_state) r = max_sync(c);  // the replaced state's pending end state
  if (!r) {
    c->max_pending = false;
    c->max_fresh = true;
    c->cur = 0;
    ++c->launches;
    k_init_state<<<grid2(c->pitch, c->ny), 128, 0, c->stream>>>(
        c->nx, c->ny, c->pitch, dsrc, is_cel, dx, dy, c->dep, c->dep64, c->srf[0], c->xu[0], c->yv[0], c->ground,
        kGrav);
    if (cudaGetLastError() != cudaSuccess) r = CLIFFS_ERR_CUDA;
  }
  if (!r && reset_max) {
    ++c->launches;
    k_reset_max<<<grid2(c->pitch, c->ny), 128, 0, c->stream>>>(c->nx, c->ny, c->pitch, c->dep, c->hmax, c->velmax);
    if (cudaGetLastError() != cudaSuccess) r = CLIFFS_ERR_CUDA;
  }
  // the caller's arrays are read before the call returns
  if (cudaStreamSynchronize(c->stream) != cudaSuccess && !r) r = CLIFFS_ERR_CUDA;
  if (!r) c->have_state = true;
  return r;
}

int cliffs_gpu_set_initial(cliffs_ctx* c, const double* H, const double* xv, const double* yv) {
  return upload_common(c, H, 0, xv, yv, true);
}

int cliffs_gpu_upload_state(cliffs_ctx* c, const double* cel, const double* xv, const double* yv) {
  if (c && !c->have_state) {
    int r = upload_common(c, cel, 1, xv, yv, true);
    return r;
  }
  return upload_common(c, cel, 1, xv, yv, false);
}

int cliffs_gpu_download_state(cliffs_ctx* c, double* cel, double* xv, double* yv) {
  if (!c) return CLIFFS_ERR_ARG;
  if (!c->have_state) return CLIFFS_ERR_STATE;
  const size_t n = (size_t)c->nx * c->ny;
  double *mc = (double*)host_mapped(cel, c->dev), *mx = (double*)host_mapped(xv, c->dev),
         *my = (double*)host_mapped(yv, c->dev);
  const bool direct = (!cel || mc) && (!xv || mx) && (!yv || my);  // pinned: converted in place
  double* x = nullptr;
  if (!direct) RET(xfer_area(c, &x));
  double *a = direct ? mc : (cel ? x : nullptr), *b = direct ? mx : (xv ? x + n : nullptr),
         *e = direct ? my : (yv ? x + 2 * n : nullptr);
  int r = CLIFFS_OK;
  ++c->launches;
  k_download<<<grid2(c->nx, c->ny), 128, 0, c->stream>>>(c->nx, c->ny, c->pitch, c->dep, c->dep64,
                                                        c->srf[c->cur], c->xu[c->cur], c->yv[c->cur], a, b, e,
                                                        kGrav);
  if (cudaGetLastError() != cudaSuccess) r = CLIFFS_ERR_CUDA;
  if (!direct) {
    if (!r && cel && cudaMemcpyAsync(cel, a, n * 8, cudaMemcpyDeviceToHost, c->stream)) r = CLIFFS_ERR_CUDA;
    if (!r && xv && cudaMemcpyAsync(xv, b, n * 8, cudaMemcpyDeviceToHost, c->stream)) r = CLIFFS_ERR_CUDA;
    if (!r && yv && cudaMemcpyAsync(yv, e, n * 8, cudaMemcpyDeviceToHost, c->stream)) r = CLIFFS_ERR_CUDA;
  }
  if (cudaStreamSynchronize(c->stream) != cudaSuccess && !r) r = CLIFFS_ERR_CUDA;
  return r;
}

namespace {

// The bottom rises by q (device, pitched FP32) under the standing water
// column (cliffs_main.f:205-208): the FP64 depth the context keeps moves, the
// FP32 depth becomes its rounding.  Synchronises.
int move_bottom(cliffs_ctx* c, const float* q) {
  ++c->launches;
  k_move_bottom64<<<grid2(c->nx, c->ny), 128, 0, c->stream>>>(c->nx, c->ny, c->pitch, q, c->dep64, c->dep,
                                                              c->srf[c->cur]);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(c->stream));
  return CLIFFS_OK;
}

}  // namespace

int cliffs_gpu_add_source(cliffs_ctx* c, const double* xcrd, const double* ycrd, const cliffs_source* src) {
  if (!c || !xcrd || !ycrd || !src) return CLIFFS_ERR_ARG;
  if (!c->have_state) return CLIFFS_ERR_STATE;
  if (!(src->ax > 0) || !(src->ay > 0) || !(src->rise_time >= 0) || !std::isfinite(src->amp) ||
      !std::isfinite(src->dipole) || (src->bottom && src->rise_time > 0) || c->rise_on)
    return CLIFFS_ERR_ARG;
  RET(max_sync(c));
  if (src->rise_time == 0) c->max_fresh = true;  // the state changes outside a step
  const size_t cells = (size_t)c->pitch * c->ny;
  double *dx = nullptr, *dy = nullptr;
  float* q = nullptr;
  int r = CLIFFS_OK;
  if (dalloc(&dx, (size_t)c->nx) || dalloc(&dy, (size_t)c->ny) || dalloc(&q, cells)) r = CLIFFS_ERR_NOMEM;
  if (!r && (cudaMemcpyAsync(dx, xcrd, c->nx * sizeof(double), cudaMemcpyHostToDevice, c->stream) ||
             cudaMemcpyAsync(dy, ycrd, c->ny * sizeof(double), cudaMemcpyHostToDevice, c->stream)))
    r = CLIFFS_ERR_CUDA;
  SourceParams S{src->x0, src->y0, src->ax, src->ay, cos(src->angle), sin(src->angle), src->amp, src->dipole};
  if (!r) {
    ++c->launches;
    k_source<<<grid2(c->pitch, c->ny), 128, 0, c->stream>>>(c->nx, c->ny, c->pitch, dx, dy, S, q);
    if (cudaGetLastError() != cudaSuccess) r = CLIFFS_ERR_CUDA;
  }
  if (!r && src->bottom) {
    r = move_bottom(c, q);
  } else if (!r && src->rise_time == 0) {
    ++c->launches;
    k_add_surface<<<grid2(c->nx, c->ny), 128, 0, c->stream>>>(c->nx, c->ny, c->pitch, c->dep, c->srf[c->cur], q,
                                                              1.f, 0.f, (float)c->ground);
    if (cudaGetLastError() != cudaSuccess) r = CLIFFS_ERR_CUDA;
  } else if (!r) {  // applied step by step from now on
    std::swap(c->rise_q, q);
    c->rise_T = src->rise_time;
    c->rise_el = 0;
    c->rise_w = 0;
    c->rise_on = true;
  }
  if (cudaStreamSynchronize(c->stream) != cudaSuccess && !r) r = CLIFFS_ERR_CUDA;
  cudaFree(dx);
  cudaFree(dy);
  if (q) cudaFree(q);
  return r;
}

namespace {

// NestedGrid.f:129-148: the 1-based ip with xx(ip) <= xp <= xx(ip+1) by
// bisection, and the weight of xx(ip).
void pinpoint_host(const double* xx, int n, double xp, int32_t* ip_out, double* cp) {
  int ip = 1, ipp = n;
  while (ip + 2 <= ipp) {
    const int med = (ip + ipp) / 2;
    if (xp > xx[med - 1])
      ip = med;
    else
      ipp = med;
  }
  *ip_out = ip;
  *cp = n > 1 ? (xx[ip] - xp) / (xx[ip] - xx[ip - 1]) : 0.5;
}

}  // namespace

int cliffs_gpu_apply_lattice(cliffs_ctx* c, const double* xcrd, const double* ycrd, int32_t nxq, int32_t nyq,
                             const double* xq, const double* yq, const double* q, int32_t target) {
  if (!c || !xcrd || !ycrd || !q || nxq < 1 || nyq < 1 || (nxq > 1 && !xq) || (nyq > 1 && !yq)) return CLIFFS_ERR_ARG;
  if (target < CLIFFS_LATTICE_SURFACE || target > CLIFFS_LATTICE_YVEL) return CLIFFS_ERR_ARG;
  if (!c->have_state) return CLIFFS_ERR_STATE;
  if (c->rise_on) return CLIFFS_ERR_STATE;  // a source still rising owns the surface
  // apply_initial_conditions.f: lattices narrower than 3 nodes along both
  // axes, or 2 along one, leave the field as it is
  if (!((nxq > 2 && nyq > 2) || (nyq == 1 && nxq > 2) || (nxq == 1 && nyq > 2))) return CLIFFS_OK;
  for (int k = 1; k < nxq; ++k)
    if (!(xq[k] > xq[k - 1])) return CLIFFS_ERR_ARG;
  for (int k = 1; k < nyq; ++k)
    if (!(yq[k] > yq[k - 1])) return CLIFFS_ERR_ARG;
  RET(max_sync(c));
  c->max_fresh = true;  // the state changes outside a step
  // the grid's columns and rows in the lattice, on the host (O(nx + ny))
  const double zero = 0.1e-20;
  std::vector<int32_t> ii(c->nx, -1), jj(c->ny, -1);
  std::vector<double> xc(c->nx, 0.0), yc(c->ny, 0.0);
  if (nxq > 2) {
    const double x1 = xq[0] - zero, x2 = xq[nxq - 1] + zero;
    for (int i = 0; i < c->nx; ++i)
      if (xcrd[i] >= x1 && xcrd[i] <= x2) pinpoint_host(xq, nxq, xcrd[i], &ii[i], &xc[i]);
  }
  if (nyq > 2) {
    const double y1 = yq[0] - zero, y2 = yq[nyq - 1] + zero;
    for (int j = 0; j < c->ny; ++j)
      if (ycrd[j] >= y1 && ycrd[j] <= y2) pinpoint_host(yq, nyq, ycrd[j], &jj[j], &yc[j]);
  }
  const size_t cells = (size_t)c->pitch * c->ny;
  int32_t *dii = nullptr, *djj = nullptr;
  double *dxc = nullptr, *dyc = nullptr, *dq = nullptr;
  float* f = nullptr;
  int r = CLIFFS_OK;
  if (dalloc(&dii, (size_t)c->nx) || dalloc(&djj, (size_t)c->ny) || dalloc(&dxc, (size_t)c->nx) ||
      dalloc(&dyc, (size_t)c->ny) || dalloc(&dq, (size_t)nxq * nyq) || dalloc(&f, cells))
    r = CLIFFS_ERR_NOMEM;
  if (!r && (cudaMemcpy(dii, ii.data(), c->nx * 4, cudaMemcpyHostToDevice) ||
             cudaMemcpy(djj, jj.data(), c->ny * 4, cudaMemcpyHostToDevice) ||
             cudaMemcpy(dxc, xc.data(), c->nx * 8, cudaMemcpyHostToDevice) ||
             cudaMemcpy(dyc, yc.data(), c->ny * 8, cudaMemcpyHostToDevice) ||
             cudaMemcpy(dq, q, (size_t)nxq * nyq * 8, cudaMemcpyHostToDevice)))
    r = CLIFFS_ERR_CUDA;
  if (!r) {
    ++c->launches;
    k_lattice<<<grid2(c->pitch, c->ny), 128, 0, c->stream>>>(c->nx, c->ny, c->pitch, dii, dxc, djj, dyc, nxq, nyq,
                                                              dq, f);
    if (cudaGetLastError() != cudaSuccess) r = CLIFFS_ERR_CUDA;
  }
  if (!r) {
    if (target == CLIFFS_LATTICE_BOTTOM) {
      r = move_bottom(c, f);
    } else if (target == CLIFFS_LATTICE_SURFACE) {
      ++c->launches;
      k_add_surface<<<grid2(c->nx, c->ny), 128, 0, c->stream>>>(c->nx, c->ny, c->pitch, c->dep, c->srf[c->cur], f,
                                                                1.f, 0.f, (float)c->ground);
      if (cudaGetLastError() != cudaSuccess) r = CLIFFS_ERR_CUDA;
    } else {
      ++c->launches;
      float* u = target == CLIFFS_LATTICE_XVEL ? c->xu[c->cur] : c->yv[c->cur];
      k_add_field<<<grid2(c->nx, c->ny), 128, 0, c->stream>>>(c->nx, c->ny, c->pitch, u, f);
      if (cudaGetLastError() != cudaSuccess) r = CLIFFS_ERR_CUDA;
    }
  }
  if (cudaStreamSynchronize(c->stream) != cudaSuccess && !r) r = CLIFFS_ERR_CUDA;
  for (void* p : {(void*)dii, (void*)djj, (void*)dxc, (void*)dyc, (void*)dq, (void*)f})
    if (p) cudaFree(p);
  return r;
}

int cliffs_depth_ssl(int32_t nx, int32_t ny, double* dep, double alpha, double depmin, int32_t* counts,
                     int32_t* status) {
  if (nx < 1 || ny < 1 || !dep || !counts || !status || !(alpha > 0) || !(depmin > 0)) return CLIFFS_ERR_ARG;
  int dev = 0;
  int r = check_device(&dev);
  if (r) return r;
  const size_t n = (size_t)nx * ny;
  double* b = nullptr;
  unsigned* cnt = nullptr;
  if (dalloc(&b, n) || dalloc(&cnt, 1)) {
    if (b) cudaFree(b);
    return CLIFFS_ERR_NOMEM;
  }
  for (int k = 0; k < 24; ++k) counts[k] = 0;
  *status = 0;
  const double alp2 = alpha * alpha;
  auto passage = [&](int phase, unsigned* nodes) {
    if (cudaMemset(cnt, 0, sizeof(unsigned)) != cudaSuccess) return CLIFFS_ERR_CUDA;
    if (phase == 0) {
      k_depth_ssl<0, 0><<<(nx + 127) / 128, 128>>>(nx, ny, b, alpha, alp2, depmin, cnt);
      k_depth_ssl<0, 1><<<(ny + 127) / 128, 128>>>(nx, ny, b, alpha, alp2, depmin, cnt);
    } else {
      k_depth_ssl<1, 0><<<(nx + 127) / 128, 128>>>(nx, ny, b, alpha, alp2, depmin, cnt);
      k_depth_ssl<1, 1><<<(ny + 127) / 128, 128>>>(nx, ny, b, alpha, alp2, depmin, cnt);
    }
    if (cudaGetLastError() != cudaSuccess) return CLIFFS_ERR_CUDA;
    if (cudaMemcpy(nodes, cnt, sizeof(unsigned), cudaMemcpyDeviceToHost) != cudaSuccess) return CLIFFS_ERR_CUDA;
    return CLIFFS_OK;
  };
  if (cudaMemcpy(b, dep, n * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess) r = CLIFFS_ERR_CUDA;
  // up to 12 passages per phase, each ending early once no node moves
  for (int phase = 0; phase < 2 && !r; ++phase) {
    unsigned nodes = 0;
    for (int itry = 0; itry < 12 && !r; ++itry) {
      r = passage(phase, &nodes);
      if (r) break;
      counts[12 * phase + itry] = (int32_t)nodes;
      if (nodes == 0) break;
    }
    if (!r && nodes != 0) *status |= 1 << phase;
  }
  if (!r && cudaMemcpy(dep, b, n * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess) r = CLIFFS_ERR_CUDA;
  cudaFree(b);
  cudaFree(cnt);
  return r;
}

int cliffs_boundary_scan(int32_t nx, int32_t ny, int32_t nt, const float* cube, double cuke, int32_t* first) {
  if (nx < 1 || ny < 1 || nt < 1 || !cube || !first) return CLIFFS_ERR_ARG;
  int dev = 0;
  int r = check_device(&dev);
  if (r) return r;
  const size_t n = (size_t)nx * ny * nt;
  float *d = nullptr, *hi = nullptr, *lo = nullptr;
  if (dalloc(&d, n) || dalloc(&hi, (size_t)nt) || dalloc(&lo, (size_t)nt)) r = CLIFFS_ERR_NOMEM;
  std::vector<float> h(nt), l(nt);
  if (!r && cudaMemcpy(d, cube, n * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess) r = CLIFFS_ERR_CUDA;
  if (!r) {
    k_boundary_scan<<<nt, 256>>>(nx, ny, d, hi, lo);
    if (cudaGetLastError() != cudaSuccess || cudaMemcpy(h.data(), hi, nt * 4, cudaMemcpyDeviceToHost) ||
        cudaMemcpy(l.data(), lo, nt * 4, cudaMemcpyDeviceToHost))
      r = CLIFFS_ERR_CUDA;
  }
  if (!r) {  // scan4wave.f: the first record above cuke, nt + 1 when none
    int it = 1;
    while (it <= nt && !((double)h[it - 1] > cuke || (double)l[it - 1] > cuke)) ++it;
    *first = it;
  }
  for (void* p : {(void*)d, (void*)hi, (void*)lo})
    if (p) cudaFree(p);
  return r;
}

int cliffs_boundary_edges(const cliffs_nest_desc* t, int32_t nx, int32_t ny, int32_t nt, const float* cube,
                          double scale, int32_t ival, double* west, double* east, double* south, double* north) {
  if (!t || !cube || !west || !east || !south || !north || nx < 2 || ny < 2 || nt < 1 || ival < 1 || ival > 3 ||
      t->mm < 1 || t->nn < 1 || !t->WE_ny || !t->WE_cy || !t->SN_nx || !t->SN_cx)
    return CLIFFS_ERR_ARG;
  // every lattice column and row the interpolation reads lies in the cube
  for (int i = 0; i < t->nn; ++i) {
    const int kk = t->WE_ny[i] - t->WE_ny[0] + 1;
    if (kk < 1 || kk + 1 > ny) return CLIFFS_ERR_ARG;
  }
  for (int i = 0; i < t->mm; ++i) {
    const int kk = t->SN_nx[i] - t->SN_nx[0] + 1;
    if (kk < 1 || kk + 1 > nx) return CLIFFS_ERR_ARG;
  }
  int dev = 0;
  int r = check_device(&dev);
  if (r) return r;
  const int mm = t->mm, nn = t->nn;
  const size_t n = (size_t)nx * ny * nt, rw = (size_t)3 * nn * nt, rs = (size_t)3 * mm * nt;
  float* d = nullptr;
  int32_t *we = nullptr, *sn = nullptr;
  double *wc = nullptr, *sc = nullptr, *out = nullptr;
  if (dalloc(&d, n) || dalloc(&we, (size_t)nn) || dalloc(&sn, (size_t)mm) || dalloc(&wc, (size_t)nn) ||
      dalloc(&sc, (size_t)mm) || dalloc(&out, 2 * rw + 2 * rs))
    r = CLIFFS_ERR_NOMEM;
  double *dw = out, *de = out + rw, *ds = out + 2 * rw, *dn = out + 2 * rw + rs;
  // the other components of the records stay as the caller has them
  if (!r && (cudaMemcpy(d, cube, n * 4, cudaMemcpyHostToDevice) || cudaMemcpy(we, t->WE_ny, nn * 4, cudaMemcpyHostToDevice) ||
             cudaMemcpy(sn, t->SN_nx, mm * 4, cudaMemcpyHostToDevice) ||
             cudaMemcpy(wc, t->WE_cy, nn * 8, cudaMemcpyHostToDevice) ||
             cudaMemcpy(sc, t->SN_cx, mm * 8, cudaMemcpyHostToDevice) ||
             cudaMemcpy(dw, west, rw * 8, cudaMemcpyHostToDevice) || cudaMemcpy(de, east, rw * 8, cudaMemcpyHostToDevice) ||
             cudaMemcpy(ds, south, rs * 8, cudaMemcpyHostToDevice) ||
             cudaMemcpy(dn, north, rs * 8, cudaMemcpyHostToDevice)))
    r = CLIFFS_ERR_CUDA;
  if (!r) {
    const long long work = (long long)(nn + mm) * nt;
    k_boundary_edges<<<(unsigned)((work + 127) / 128), 128>>>(nx, ny, nt, d, (float)scale, ival, mm, nn, t->W_cx,
                                                               t->E_cx, t->S_cy, t->N_cy, we, wc, sn, sc, dw, de, ds,
                                                               dn);
    if (cudaGetLastError() != cudaSuccess || cudaMemcpy(west, dw, rw * 8, cudaMemcpyDeviceToHost) ||
        cudaMemcpy(east, de, rw * 8, cudaMemcpyDeviceToHost) || cudaMemcpy(south, ds, rs * 8, cudaMemcpyDeviceToHost) ||
        cudaMemcpy(north, dn, rs * 8, cudaMemcpyDeviceToHost))
      r = CLIFFS_ERR_CUDA;
  }
  for (void* p : {(void*)d, (void*)we, (void*)sn, (void*)wc, (void*)sc, (void*)out})
    if (p) cudaFree(p);
  return r;
}

int cliffs_gpu_set_feed(cliffs_ctx* c, int32_t nt, const double* tinput, const double* west,
                        const double* east, const double* south, const double* north, int32_t irec,
                        int32_t freeze) {
  if (!c) return CLIFFS_ERR_ARG;
  CK(cudaStreamSynchronize(c->stream));
  if (c->fgraph) {  // captured with the records being replaced
    cudaGraphExecDestroy(c->fgraph);
    c->fgraph = nullptr;
  }
  double** bufs[] = {&c->fw, &c->fe, &c->fs, &c->fn};
  for (double** b : bufs)
    if (*b) {
      cudaFree(*b);
      *b = nullptr;
    }
  c->nt = 0;
  c->feed_on = false;
  c->tinput.clear();
  if (nt == 0) return CLIFFS_OK;
  if (nt < 2 || !tinput || irec < 1 || irec > nt) return CLIFFS_ERR_ARG;
  if (c->xrun && (!west || !east)) return CLIFFS_ERR_ARG;
  if (c->yrun && (!south || !north)) return CLIFFS_ERR_ARG;
  c->tinput.assign(tinput, tinput + nt);
  const size_t nxr = (size_t)c->ny * 3 * nt, nyr = (size_t)c->nx * 3 * nt;
  if (c->xrun) {
    if (dalloc(&c->fw, nxr) || dalloc(&c->fe, nxr)) return CLIFFS_ERR_NOMEM;
    CK(cudaMemcpy(c->fw, west, nxr * 8, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(c->fe, east, nxr * 8, cudaMemcpyHostToDevice));
  }
  if (c->yrun) {
    if (dalloc(&c->fs, nyr) || dalloc(&c->fn, nyr)) return CLIFFS_ERR_NOMEM;
    CK(cudaMemcpy(c->fs, south, nyr * 8, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(c->fn, north, nyr * 8, cudaMemcpyHostToDevice));
  }
  c->nt = nt;
  c->irec = irec;
  c->freeze = freeze != 0;
  c->feed_on = true;
  return CLIFFS_OK;
}

int cliffs_gpu_feed_start(cliffs_ctx* c, double cuke) {
  // get_boundary_feed.f:144-167, on the host copy of the records
  if (!c || c->nt < 2) return CLIFFS_ERR_ARG;
  const int nt = c->nt;
  std::vector<double> w, e, s, n;
  const size_t nxr = (size_t)c->ny * 3 * nt, nyr = (size_t)c->nx * 3 * nt;
  if (c->xrun) {
    w.resize(nxr);
    e.resize(nxr);
    if (cudaMemcpy(w.data(), c->fw, nxr * 8, cudaMemcpyDeviceToHost) ||
        cudaMemcpy(e.data(), c->fe, nxr * 8, cudaMemcpyDeviceToHost))
      return CLIFFS_ERR_CUDA;
  }
  if (c->yrun) {
    s.resize(nyr);
    n.resize(nyr);
    if (cudaMemcpy(s.data(), c->fs, nyr * 8, cudaMemcpyDeviceToHost) ||
        cudaMemcpy(n.data(), c->fn, nyr * 8, cudaMemcpyDeviceToHost))
      return CLIFFS_ERR_CUDA;
  }
  auto amp = [](const double* a, int len) {
    double mx = a[0], mn = a[0];
    for (int k = 1; k < len; ++k) {
      mx = std::max(mx, a[k]);
      mn = std::min(mn, a[k]);
    }
    return mx > -mn ? mx : -mn;
  };
  double w1 = 0, w2 = 0, w3 = 0, w4 = 0;
  int it;
  for (it = 1; it <= nt; ++it) {
    if (c->xrun) {
      const size_t o = (size_t)c->ny * 2 + (size_t)(it - 1) * c->ny * 3;
      w1 = amp(w.data() + o, c->ny);
      w2 = amp(e.data() + o, c->ny);
    }
    if (c->yrun) {
      const size_t o = (size_t)c->nx * 2 + (size_t)(it - 1) * c->nx * 3;
      w3 = amp(s.data() + o, c->nx);
      w4 = amp(n.data() + o, c->nx);
    }
    const double wave = std::max(std::max(w1, w2), std::max(w3, w4));
    if (wave >= cuke) break;
  }
  return it >= nt ? -1 : it;
}

// Forced steps of a two-dimensional grid from a CUDA graph of graph_k steps:
// the host advances the forcing record cursor for the chunk exactly as
// one_step does, copies each step's record and weight to the device, and the
// graph computes all the chunk's edge tables in one kernel (edges_ring_kernel)
// before its 2 * graph_k sweeps, each reading its own table.  A chunk in
// which the forcing ends is left to one_step.
static int forced_graph_steps(cliffs_ctx* c, int nsteps, double* t, int32_t* steps_done, int* done_out) {
  const int k = c->graph_k;
  *done_out = 0;
  if (!c->feed_on || k < 2 || nsteps < k || c->prof || c->rise_on || c->max_fresh || !c->xrun || !c->yrun)
    return CLIFFS_OK;
  if (c->ring_k != k) {
    for (void* p : {(void*)c->ring_x, (void*)c->ring_y, (void*)c->ring_irec, (void*)c->ring_cc})
      if (p) cudaFree(p);
    c->ring_x = c->ring_y = nullptr;
    c->ring_irec = nullptr;
    c->ring_cc = nullptr;
    c->ring_k = 0;
    if (c->ring_host) {
      CK(cudaStreamSynchronize(c->stream));  // no copy from the old slots is pending
      cudaFreeHost(c->ring_host);
      c->ring_host = nullptr;
    }
    if (dalloc(&c->ring_x, (size_t)k * 6 * c->ny) || dalloc(&c->ring_y, (size_t)k * 6 * c->nx) ||
        dalloc(&c->ring_irec, (size_t)k) || dalloc(&c->ring_cc, (size_t)k) ||
        cudaHostAlloc((void**)&c->ring_host, (size_t)cliffs_ctx::kRingSlots * k * 16, cudaHostAllocDefault) !=
            cudaSuccess)
      return CLIFFS_ERR_NOMEM;
    for (cudaEvent_t& e : c->ring_ev)
      if (!e && cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return CLIFFS_ERR_CUDA;
    c->ring_k = k;
    if (c->fgraph) cudaGraphExecDestroy(c->fgraph);
    c->fgraph = nullptr;
  }
  if (!c->fgraph || c->fgraph_k != k || c->fgraph_cur != c->cur || c->fgraph_blk != c->blk_x ||
      c->fgraph_wy != c->warps_y || c->fgraph_kind != c->sweep_kind) {
    if (c->fgraph) cudaGraphExecDestroy(c->fgraph);
    c->fgraph = nullptr;
    const int64_t launches = c->launches;
    const unsigned sweeps = c->sweeps;
    const bool pending = c->max_pending, fresh = c->max_fresh;
    cudaGraph_t g = nullptr;
    CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    const long long work = (long long)(c->nx + c->ny) * k;
    edges_ring_kernel<<<(unsigned)((work + 127) / 128), 128, 0, c->stream>>>(
        k, c->nx, c->ny, c->fw, c->fe, c->fs, c->fn, c->ring_irec, c->ring_cc, c->ring_x, c->ring_y);
    int r = cudaGetLastError() == cudaSuccess ? CLIFFS_OK : CLIFFS_ERR_CUDA;
    for (int s = 0; s < k && !r; ++s) {  // every step alike: the state is not fresh here
      int mx, my;
      step_modes(c, &mx, &my);
      r = launch_sweep(c, 1, mx, c->fw, c->fe, c->ny, 2, 0.0, c->ring_x + (size_t)s * 6 * c->ny);
      if (!r) r = launch_sweep(c, 2, my, c->fs, c->fn, c->nx, 2, 0.0, c->ring_y + (size_t)s * 6 * c->nx);
      step_done(c);
    }
    const cudaError_t e = cudaStreamEndCapture(c->stream, &g);
    c->launches = launches;  // captured, not launched
    c->sweeps = sweeps;
    c->max_pending = pending;
    c->max_fresh = fresh;
    if (r || e != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      return r ? r : CLIFFS_ERR_CUDA;
    }
    const cudaError_t ie = cudaGraphInstantiate(&c->fgraph, g, 0);
    cudaGraphDestroy(g);
    if (ie != cudaSuccess) return CLIFFS_ERR_CUDA;
    c->fgraph_k = k;
    c->fgraph_cur = c->cur;
    c->fgraph_blk = c->blk_x;
    c->fgraph_wy = c->warps_y;
    c->fgraph_kind = c->sweep_kind;
  }
  int done = 0;
  while (done + k <= nsteps) {
    // a free pinned slot: its previous copy has completed
    const int slot = c->ring_slot;
    CK(cudaEventSynchronize(c->ring_ev[slot]));
    double* hcc = reinterpret_cast<double*>(c->ring_host + (size_t)slot * k * 16);
    int32_t* hir = reinterpret_cast<int32_t*>(c->ring_host + (size_t)slot * k * 16 + (size_t)k * 8);
    // the cursor of cliffs_main.f:305-315 over the chunk, as one_step runs it
    double tt = *t;
    int ir = c->irec;
    bool regular = true;
    for (int s = 0; s < k && regular; ++s) {
      tt = tt + c->dt;
      while (tt >= c->tinput[ir - 1]) {
        if (ir == c->nt) {
          regular = false;
          break;
        }
        ir = ir + 1;
      }
      if (!regular) break;
      hir[s] = ir;
      hcc[s] = (c->tinput[ir - 1] - tt) / (c->tinput[ir - 1] - c->tinput[ir - 2]);
    }
    if (!regular) break;  // the forcing ends in this chunk
    CK(cudaMemcpyAsync(c->ring_irec, hir, (size_t)k * sizeof(int32_t), cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->ring_cc, hcc, (size_t)k * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    CK(cudaEventRecord(c->ring_ev[slot], c->stream));
    c->ring_slot = (slot + 1) % cliffs_ctx::kRingSlots;
    CK(cudaGraphLaunch(c->fgraph, c->stream));
    c->launches += 1 + 2 * (int64_t)k;
    c->sweeps += 2u * (unsigned)k;
    *t = tt;
    c->irec = ir;
    for (int s = 0; s < k; ++s) step_done(c);
    if (steps_done) *steps_done += k;
    done += k;
  }
  *done_out = done;
  return CLIFFS_OK;
}

// Plain steps (no forcing, profiling or rising source) from CUDA graphs: one
// launch per graph_k steps instead of two per step, and the remaining steps
// of a call (at least 2) from a graph of their own length.  A whole step
// leaves the state copy where it found it, so a graph's arguments hold for
// every replay.  Every captured step folds the previous step's end state
// into the max-wave fields (the state is not fresh).
static bool plain_graph_valid(const cliffs_ctx* c, const cliffs_ctx::PlainGraph& pg, int len) {
  return pg.exec && pg.len == len && pg.cur == c->cur && pg.blk == c->blk_x && pg.wy == c->warps_y &&
         pg.kind == c->sweep_kind;
}

static int plain_graph(cliffs_ctx* c, int len, cliffs_ctx::PlainGraph** out) {
  *out = nullptr;
  const bool full = len == c->graph_k;
  int slot = 0;
  if (!full) {  // a tail: the slot that holds this length, else the oldest
    slot = 1;
    for (int s = 1; s < cliffs_ctx::kPlainGraphs; ++s) {
      if (plain_graph_valid(c, c->pgraph[s], len)) {
        slot = s;
        break;
      }
      if (c->pgraph[s].used < c->pgraph[slot].used) slot = s;
    }
  }
  cliffs_ctx::PlainGraph& pg = c->pgraph[slot];
  pg.used = ++c->pgraph_clock;
  if (plain_graph_valid(c, pg, len)) {
    *out = &pg;
    return CLIFFS_OK;
  }
  if (pg.exec) cudaGraphExecDestroy(pg.exec);
  pg = cliffs_ctx::PlainGraph{};
  pg.used = c->pgraph_clock;
  const int64_t launches = c->launches;
  const unsigned sweeps = c->sweeps;
  const bool fresh = c->max_fresh, pending = c->max_pending;
  const int cur = c->cur;
  c->max_fresh = false;  // every captured step folds in the previous one
  cudaGraph_t g = nullptr;
  CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
  int r = CLIFFS_OK;
  for (int s = 0; s < len && !r; ++s) {
    int mx, my;
    step_modes(c, &mx, &my);
    if (c->xrun) r = launch_sweep(c, 1, mx, nullptr, nullptr, c->ny, 2, 0.0);
    if (!r && c->yrun) r = launch_sweep(c, 2, my, nullptr, nullptr, c->nx, 2, 0.0);
    step_done(c);
  }
  const cudaError_t e = cudaStreamEndCapture(c->stream, &g);
  // captured, not launched: the bookkeeping is the caller's, per replay
  c->launches = launches;
  c->sweeps = sweeps;
  c->max_fresh = fresh;
  c->max_pending = pending;
  c->cur = cur;
  if (r || e != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    return r ? r : CLIFFS_ERR_CUDA;
  }
  const cudaError_t ie = cudaGraphInstantiate(&pg.exec, g, 0);
  cudaGraphDestroy(g);
  if (ie != cudaSuccess) {
    pg.exec = nullptr;
    return CLIFFS_ERR_CUDA;
  }
  pg.len = len;
  pg.cur = c->cur;
  pg.blk = c->blk_x;
  pg.wy = c->warps_y;
  pg.kind = c->sweep_kind;
  *out = &pg;
  return CLIFFS_OK;
}

static bool plain_graphs_apply(const cliffs_ctx* c) {
  return c->graph_k >= 2 && !c->feed_on && !c->prof && !c->rise_on;
}

// Steps of the next graph for `remaining` steps: graph_k, or the rest; a
// one-dimensional grid (one sweep per step) takes an even count, so that a
// graph ends on the state copy it started from.  0: none (run directly).
static int plain_graph_len(const cliffs_ctx* c, int remaining) {
  const int per = (c->xrun ? 1 : 0) + (c->yrun ? 1 : 0);
  int len = std::min(c->graph_k, remaining);
  if ((per * len) & 1) len -= 1;
  return len >= 2 ? len : 0;
}

// The instantiated graph of `len` steps for the current state copy and
// tiling, or nullptr.
static cliffs_ctx::PlainGraph* plain_graph_find(cliffs_ctx* c, int len) {
  for (int s = 0; s < cliffs_ctx::kPlainGraphs; ++s)
    if (plain_graph_valid(c, c->pgraph[s], len)) {
      c->pgraph[s].used = ++c->pgraph_clock;
      return &c->pgraph[s];
    }
  return nullptr;
}

static int one_step(cliffs_ctx* c, double* t);

static int graph_steps(cliffs_ctx* c, int nsteps, double* t, int32_t* steps_done, int* done_out) {
  *done_out = 0;
  if (!plain_graphs_apply(c) || nsteps < 2) return CLIFFS_OK;
  const int per = (c->xrun ? 1 : 0) + (c->yrun ? 1 : 0);
  int done = 0;
  for (int len; (len = plain_graph_len(c, nsteps - done)) > 0;) {
    cliffs_ctx::PlainGraph* pg = plain_graph_find(c, len);
    if (!pg) {
      // no graph of this length yet: these steps run launch by launch, and
      // the graph is captured and instantiated while the device works on
      // them, for the calls that follow (cliffs_gpu_prepare_steps builds it
      // ahead instead)
      for (int s = 0; s < len; ++s) {
        RET(one_step(c, t));
        if (steps_done) *steps_done += 1;
      }
      RET(plain_graph(c, len, &pg));
      done += len;
      continue;
    }
    CK(cudaGraphLaunch(pg->exec, c->stream));
    c->launches += (int64_t)per * len;
    c->sweeps += (unsigned)(per * len);
    for (int s = 0; s < len; ++s) step_done(c);
    for (int s = 0; s < len; ++s) *t = *t + c->dt;
    if (steps_done) *steps_done += len;
    done += len;
  }
  *done_out = done;
  return CLIFFS_OK;
}

int cliffs_gpu_prepare_steps(cliffs_ctx* c, int32_t nsteps) {
  if (!c || nsteps < 0) return CLIFFS_ERR_ARG;
  if (!c->have_state) return CLIFFS_ERR_STATE;
  if (!plain_graphs_apply(c)) return CLIFFS_OK;
  // the graphs cliffs_gpu_step(nsteps) would replay; a fresh state's first
  // step runs alone
  int n = nsteps - (c->max_fresh && nsteps > 0 ? 1 : 0);
  int last = -1;
  for (int len; (len = plain_graph_len(c, n)) > 0; n -= len) {
    if (len == last) continue;
    cliffs_ctx::PlainGraph* pg = nullptr;
    RET(plain_graph(c, len, &pg));
    last = len;
  }
  return CLIFFS_OK;
}

int cliffs_gpu_set_graph_steps(cliffs_ctx* c, int32_t k) {
  if (!c || k < 0 || k > 4096) return CLIFFS_ERR_ARG;
  c->graph_k = k;
  return CLIFFS_OK;
}

// One step of the time loop body (cliffs_main.f:304-355) with a launch per
// sweep; CLIFFS_FEED_ENDED when the forcing ended with freeze (t advanced,
// nothing swept).
static int one_step(cliffs_ctx* c, double* t) {
  *t = *t + c->dt;
  // forcing record cursor (cliffs_main.f:305-315)
  while (c->feed_on && *t >= c->tinput[c->irec - 1]) {
    if (c->irec == c->nt) {
      c->feed_on = false;
      if (c->freeze) return CLIFFS_FEED_ENDED;
    } else {
      c->irec = c->irec + 1;
    }
  }
  double cc = 0;
  if (c->feed_on) cc = (c->tinput[c->irec - 1] - *t) / (c->tinput[c->irec - 1] - c->tinput[c->irec - 2]);
  if (c->rise_on) {  // the rising source's share of this step
    RET(max_sync(c));
    c->max_fresh = true;  // the surface changes before the sweeps
    c->rise_el += c->dt;
    const double w = std::min(1.0, c->rise_el / c->rise_T);
    ++c->launches;
    k_add_surface<<<grid2(c->nx, c->ny), 128, 0, c->stream>>>(c->nx, c->ny, c->pitch, c->dep, c->srf[c->cur],
                                                              c->rise_q, (float)w, (float)c->rise_w,
                                                              (float)c->ground);
    CK(cudaGetLastError());
    c->rise_w = w;
    if (w >= 1.0) c->rise_on = false;
  }
  int mx, my;
  step_modes(c, &mx, &my);
  if (c->xrun) {
    int r = launch_sweep(c, 1, mx, c->feed_on ? c->fw : nullptr, c->feed_on ? c->fe : nullptr, c->ny, c->irec, cc);
    if (r) return r;
  }
  if (c->yrun) {
    int r = launch_sweep(c, 2, my, c->feed_on ? c->fs : nullptr, c->feed_on ? c->fn : nullptr, c->nx, c->irec, cc);
    if (r) return r;
  }
  step_done(c);
  return CLIFFS_OK;
}

int cliffs_gpu_step(cliffs_ctx* c, int32_t nsteps, double* t, int32_t* steps_done) {
  if (!c || !t || nsteps < 0) return CLIFFS_ERR_ARG;
  if (!c->have_state) return CLIFFS_ERR_STATE;
  if (steps_done) *steps_done = 0;
  int done = 0;
  if (c->max_fresh && nsteps > 0) {
    // the first step from a fresh state folds nothing into the max-wave
    // fields; the graphs' steps all fold in the previous step's end state
    const int r = one_step(c, t);
    if (r) return r;
    done = 1;
    if (steps_done) *steps_done = 1;
  }
  int fdone = 0;
  const int fr = forced_graph_steps(c, nsteps - done, t, steps_done, &fdone);
  if (fr) return fr;
  done += fdone;
  int gdone = 0;
  const int gr = graph_steps(c, nsteps - done, t, steps_done, &gdone);
  if (gr) return gr;
  done += gdone;
  for (; done < nsteps; ++done) {
    const int r = one_step(c, t);
    if (r) return r;
    if (steps_done) *steps_done = done + 1;
    if (c->prof && c->prof_pending.size() > 4096) {
      const int f = flush_profile(c);
      if (f) return f;
    }
  }
  return CLIFFS_OK;
}

int cliffs_gpu_set_edges(cliffs_ctx* c, const double* edge1, const double* edge2);

int cliffs_gpu_sweep(cliffs_ctx* c, int32_t iu) {
  if (!c || (iu != 1 && iu != 2)) return CLIFFS_ERR_ARG;
  if (!c->have_state) return CLIFFS_ERR_STATE;
  if ((iu == 1 && !c->xrun) || (iu == 2 && !c->yrun)) return CLIFFS_ERR_ARG;
  const int len = iu == 1 ? c->ny : c->nx;
  RET(max_sync(c));
  c->max_fresh = true;  // a half step: not a step's end state
  if (c->edges_static) {
    // static edge1/edge2, stored as two identical records: lerp weight 1
    const int mx = std::max(c->xrun ? c->ny : 1, c->yrun ? c->nx : 1);
    (void)len;
    return launch_sweep(c, iu, MAXM_NONE, c->edge_s[0], c->edge_s[1], mx, 2, 1.0);
  }
  return launch_sweep(c, iu, MAXM_NONE, nullptr, nullptr, len, 2, 1.0);
}

int cliffs_gpu_set_edges(cliffs_ctx* c, const double* edge1, const double* edge2) {
  if (!c) return CLIFFS_ERR_ARG;
  const int mx = std::max(c->xrun ? c->ny : 1, c->yrun ? c->nx : 1);
  if (!edge1 || !edge2) {
    c->edges_static = false;
    return CLIFFS_OK;
  }
  for (int k = 0; k < 2; ++k)
    if (!c->edge_s[k] && dalloc(&c->edge_s[k], (size_t)mx * 3 * 2)) return CLIFFS_ERR_NOMEM;
  for (int k = 0; k < 2; ++k) {
    const double* src = k == 0 ? edge1 : edge2;
    CK(cudaMemcpy(c->edge_s[k], src, (size_t)mx * 3 * 8, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(c->edge_s[k] + (size_t)mx * 3, src, (size_t)mx * 3 * 8, cudaMemcpyHostToDevice));
  }
  c->edges_static = true;
  return CLIFFS_OK;
}

int cliffs_gpu_maxwave_update(cliffs_ctx* c) {
  if (!c) return CLIFFS_ERR_ARG;
  if (!c->have_state) return CLIFFS_ERR_STATE;
  c->max_pending = false;  // the update below folds the current state in
  ++c->launches;
  k_maxwave_update<<<grid2(c->nx, c->ny), 128, 0, c->stream>>>(c->nx, c->ny, c->pitch, c->dep, c->srf[c->cur],
                                                              c->xu[c->cur], c->yv[c->cur], c->hmax, c->velmax);
  CK(cudaGetLastError());
  return CLIFFS_OK;
}

int cliffs_gpu_get_maxwave(cliffs_ctx* c, float* me, float* mv) {
  if (!c || !me || !mv) return CLIFFS_ERR_ARG;
  RET(max_sync(c));
  const size_t n = (size_t)c->nx * c->ny;
  float *ma = (float*)host_mapped(me, c->dev), *mb = (float*)host_mapped(mv, c->dev);
  const bool direct = ma && mb;  // pinned: written in place
  double* x = nullptr;
  if (!direct) RET(xfer_area(c, &x));
  float *a = direct ? ma : (float*)x, *b = direct ? mb : (float*)(x + n);
  int r = CLIFFS_OK;
  ++c->launches;
  k_maxwave_out<<<grid2(c->nx, c->ny), 128, 0, c->stream>>>(c->nx, c->ny, c->pitch, c->dep, c->hmax, c->velmax,
                                                           (float)c->ground, a, b);
  if (cudaGetLastError() != cudaSuccess) r = CLIFFS_ERR_CUDA;
  if (!direct) {
    if (!r && cudaMemcpyAsync(me, a, n * 4, cudaMemcpyDeviceToHost, c->stream)) r = CLIFFS_ERR_CUDA;
    if (!r && cudaMemcpyAsync(mv, b, n * 4, cudaMemcpyDeviceToHost, c->stream)) r = CLIFFS_ERR_CUDA;
  }
  if (cudaStreamSynchronize(c->stream) != cudaSuccess && !r) r = CLIFFS_ERR_CUDA;
  return r;
}

int cliffs_gpu_get_max_raw(cliffs_ctx* c, double* hm, double* vm) {
  if (!c) return CLIFFS_ERR_ARG;
  RET(max_sync(c));
  const size_t n = (size_t)c->nx * c->ny;
  double* x = nullptr;
  RET(xfer_area(c, &x));
  double *a = x, *b = x + n;
  int r = CLIFFS_OK;
  ++c->launches;
  k_max_raw<<<grid2(c->nx, c->ny), 128, 0, c->stream>>>(c->nx, c->ny, c->pitch, c->dep, c->hmax, c->velmax, a, b,
                                                       kGrav);
  if (cudaGetLastError() != cudaSuccess) r = CLIFFS_ERR_CUDA;
  if (!r && hm && cudaMemcpyAsync(hm, a, n * 8, cudaMemcpyDeviceToHost, c->stream)) r = CLIFFS_ERR_CUDA;
  if (!r && vm && cudaMemcpyAsync(vm, b, n * 8, cudaMemcpyDeviceToHost, c->stream)) r = CLIFFS_ERR_CUDA;
  if (cudaStreamSynchronize(c->stream) != cudaSuccess && !r) r = CLIFFS_ERR_CUDA;
  return r;
}

int cliffs_gpu_get_sea_state(cliffs_ctx* c, int32_t lonsub, int32_t latsub, float* h, float* u, float* v) {
  if (!c || lonsub < 1 || latsub < 1 || !h || !u || !v) return CLIFFS_ERR_ARG;
  if (!c->have_state) return CLIFFS_ERR_STATE;
  const int nxs = (c->nx - 1) / lonsub + 1, nys = (c->ny - 1) / latsub + 1;
  const size_t n = (size_t)nxs * nys;
  float* a = nullptr;
  if (dalloc(&a, 3 * n)) return CLIFFS_ERR_NOMEM;
  int r = CLIFFS_OK;
  const int s = c->cur;
  ++c->launches;
  k_sea_state<<<grid2(nxs, nys), 128, 0, c->stream>>>(nxs, nys, c->pitch, lonsub, latsub, c->dep, c->srf[s],
                                                      c->xu[s], c->yv[s], (float)c->ground, a, a + n, a + 2 * n);
  if (cudaGetLastError() != cudaSuccess) r = CLIFFS_ERR_CUDA;
  if (!r && (cudaMemcpyAsync(h, a, n * 4, cudaMemcpyDeviceToHost, c->stream) ||
             cudaMemcpyAsync(u, a + n, n * 4, cudaMemcpyDeviceToHost, c->stream) ||
             cudaMemcpyAsync(v, a + 2 * n, n * 4, cudaMemcpyDeviceToHost, c->stream)))
    r = CLIFFS_ERR_CUDA;
  if (cudaStreamSynchronize(c->stream) != cudaSuccess && !r) r = CLIFFS_ERR_CUDA;
  cudaFree(a);
  return r;
}

int cliffs_gpu_get_gauges(cliffs_ctx* c, int32_t n, const int32_t* I, const int32_t* J, double* eta, double* u,
                          double* v) {
  if (!c || n < 0 || (n > 0 && (!I || !J || !eta || !u || !v))) return CLIFFS_ERR_ARG;
  if (!c->have_state) return CLIFFS_ERR_STATE;
  if (n == 0) return CLIFFS_OK;
  for (int k = 0; k < n; ++k)
    if (I[k] < 1 || I[k] > c->nx || J[k] < 1 || J[k] > c->ny) return CLIFFS_ERR_ARG;
  int32_t* dij = nullptr;
  double* out = nullptr;
  if (dalloc(&dij, 2 * (size_t)n) || dalloc(&out, 3 * (size_t)n)) {
    if (dij) cudaFree(dij);
    return CLIFFS_ERR_NOMEM;
  }
  int r = CLIFFS_OK;
  if (cudaMemcpyAsync(dij, I, n * 4, cudaMemcpyHostToDevice, c->stream) ||
      cudaMemcpyAsync(dij + n, J, n * 4, cudaMemcpyHostToDevice, c->stream))
    r = CLIFFS_ERR_CUDA;
  if (!r) {
    const int s = c->cur;
    ++c->launches;
    k_gauges<<<(n + 127) / 128, 128, 0, c->stream>>>(n, dij, dij + n, c->pitch, c->dep, c->srf[s], c->xu[s],
                                                     c->yv[s], (float)c->ground, out);
    if (cudaGetLastError() != cudaSuccess) r = CLIFFS_ERR_CUDA;
  }
  if (!r && (cudaMemcpyAsync(eta, out, n * 8, cudaMemcpyDeviceToHost, c->stream) ||
             cudaMemcpyAsync(u, out + n, n * 8, cudaMemcpyDeviceToHost, c->stream) ||
             cudaMemcpyAsync(v, out + 2 * n, n * 8, cudaMemcpyDeviceToHost, c->stream)))
    r = CLIFFS_ERR_CUDA;
  if (cudaStreamSynchronize(c->stream) != cudaSuccess && !r) r = CLIFFS_ERR_CUDA;
  cudaFree(dij);
  cudaFree(out);
  return r;
}

int cliffs_gpu_runup(cliffs_ctx* c, cliffs_runup* o) {
  if (!c || !o) return CLIFFS_ERR_ARG;
  if (!c->have_state) return CLIFFS_ERR_STATE;
  RET(max_sync(c));
  const int blocks = 304;
  if (c->red_cap < 4 * blocks) {
    if (c->red) cudaFree(c->red);
    c->red = nullptr;
    if (dalloc(&c->red, 4 * (size_t)blocks)) return CLIFFS_ERR_NOMEM;
    c->red_cap = 4 * blocks;
  }
  ++c->launches;
  k_runup<<<blocks, 256, 0, c->stream>>>(c->nx, c->ny, c->pitch, c->dep, c->srf[c->cur], c->hmax,
                                         (float)c->ground, c->red);
  CK(cudaGetLastError());
  std::vector<double> h(4 * (size_t)blocks);
  CK(cudaMemcpyAsync(h.data(), c->red, h.size() * 8, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  double best = -1;
  long long idx = -1, land = 0, wet = 0;
  for (int b = 0; b < blocks; ++b) {
    const double v = h[4 * b];
    const long long id = (long long)h[4 * b + 1];
    if (v > best || (v == best && id >= 0 && (idx < 0 || id < idx))) {
      best = v;
      idx = id;
    }
    land += (long long)h[4 * b + 2];
    wet += (long long)h[4 * b + 3];
  }
  o->max_runup = idx >= 0 ? best : 0.0;
  o->i = idx >= 0 ? (int32_t)(idx % c->nx) + 1 : 0;
  o->j = idx >= 0 ? (int32_t)(idx / c->nx) + 1 : 0;
  o->wetted_land = land;
  o->wet_now = wet;
  return CLIFFS_OK;
}

int cliffs_gpu_nest_add(cliffs_ctx* c, const cliffs_nest_desc* d, int32_t* id) {
  if (!c || !d || !id || d->mm < 1 || d->nn < 1 || !d->WE_ny || !d->WE_cy || !d->SN_nx || !d->SN_cx)
    return CLIFFS_ERR_ARG;
  if (!c->xrun || !c->yrun) return CLIFFS_ERR_ARG;  // allabout.f:35-39: no nesting in 1-D
  auto inside_x = [&](int i) { return i >= 1 && i + 1 <= c->nx; };
  auto inside_y = [&](int j) { return j >= 1 && j + 1 <= c->ny; };
  if (!inside_x(d->W_nx) || !inside_x(d->E_nx) || !inside_y(d->S_ny) || !inside_y(d->N_ny)) return CLIFFS_ERR_ARG;
  for (int k = 0; k < d->nn; ++k)
    if (!inside_y(d->WE_ny[k])) return CLIFFS_ERR_ARG;
  for (int k = 0; k < d->mm; ++k)
    if (!inside_x(d->SN_nx[k])) return CLIFFS_ERR_ARG;
  Nest n;
  n.d = *d;
  // footprint of the arrival test: parent rows WE_ny(1)..WE_ny(nn)+1,
  // columns SN_nx(1)..SN_nx(mm)+1
  n.k1 = d->WE_ny[0];
  n.k2 = d->WE_ny[d->nn - 1] + 1;
  n.i1 = d->SN_nx[0];
  n.i2 = d->SN_nx[d->mm - 1] + 1;
  if (dalloc(&n.WE_ny, d->nn) || dalloc(&n.WE_cy, d->nn) || dalloc(&n.SN_nx, d->mm) || dalloc(&n.SN_cx, d->mm) ||
      dalloc(&n.d_arr, 1))
    return CLIFFS_ERR_NOMEM;
  CK(cudaMemset(n.d_arr, 0, sizeof(int)));
  CK(cudaMemcpy(n.WE_ny, d->WE_ny, d->nn * 4, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(n.WE_cy, d->WE_cy, d->nn * 8, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(n.SN_nx, d->SN_nx, d->mm * 4, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(n.SN_cx, d->SN_cx, d->mm * 8, cudaMemcpyHostToDevice));
  n.d.WE_ny = nullptr;
  n.d.WE_cy = nullptr;
  n.d.SN_nx = nullptr;
  n.d.SN_cx = nullptr;
  c->nests.push_back(n);
  *id = (int32_t)c->nests.size() - 1;
  return CLIFFS_OK;
}

int cliffs_gpu_feed_child(cliffs_ctx* c, int32_t id, double cuke, int32_t* arrived, double* w, double* e,
                          double* s, double* nn_out) {
  if (!c || !arrived || id < 0 || id >= (int32_t)c->nests.size()) return CLIFFS_ERR_ARG;
  if (!c->have_state) return CLIFFS_ERR_STATE;
  const Nest& n = c->nests[id];
  const int st = c->cur;
  if (!*arrived) {
    CK(cudaMemsetAsync(c->d_flag, 0, sizeof(int), c->stream));
    ++c->launches;
    k_arrival<<<152, 256, 0, c->stream>>>(n.i1, n.i2, n.k1, n.k2, c->pitch, c->dep, c->srf[st], c->xu[st],
                                          c->yv[st], c->ground, cuke, kGrav, c->d_flag, false);
    CK(cudaGetLastError());
    int f = 0;
    CK(cudaMemcpyAsync(&f, c->d_flag, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    if (f) *arrived = 1;
  }
  if (!*arrived) return 0;
  // the asynchronous feed starts from the same arrival: the flag's low byte
  // to 1 (the int was zeroed at nest_add and only ever goes to 1)
  CK(cudaMemsetAsync(n.d_arr, 1, 1, c->stream));
  if (!w || !e || !s || !nn_out) return CLIFFS_ERR_ARG;
  const int mm = n.d.mm, nn = n.d.nn;
  double* buf = nullptr;
  if (dalloc(&buf, 6 * (size_t)(mm + nn))) return CLIFFS_ERR_NOMEM;
  double *dw = buf, *de = buf + 3 * (size_t)nn, *ds = buf + 6 * (size_t)nn, *dn = ds + 3 * (size_t)mm;
  const int threads = 2 * (mm + nn);
  ++c->launches;
  k_feed_child<<<(threads + 127) / 128, 128, 0, c->stream>>>(
      mm, nn, n.d.W_nx, n.d.E_nx, n.d.S_ny, n.d.N_ny, n.d.W_cx, n.d.E_cx, n.d.S_cy, n.d.N_cy, n.WE_ny, n.WE_cy,
      n.SN_nx, n.SN_cx, c->pitch, c->dep, c->srf[st], c->xu[st], c->yv[st], c->ground, kGrav, dw, de, ds, dn,
      nullptr, nullptr);
  int r = CLIFFS_OK;
  if (cudaGetLastError() != cudaSuccess) r = CLIFFS_ERR_CUDA;
  if (!r && (cudaMemcpyAsync(w, dw, 3 * nn * 8, cudaMemcpyDeviceToHost, c->stream) ||
             cudaMemcpyAsync(e, de, 3 * nn * 8, cudaMemcpyDeviceToHost, c->stream) ||
             cudaMemcpyAsync(s, ds, 3 * mm * 8, cudaMemcpyDeviceToHost, c->stream) ||
             cudaMemcpyAsync(nn_out, dn, 3 * mm * 8, cudaMemcpyDeviceToHost, c->stream)))
    r = CLIFFS_ERR_CUDA;
  if (cudaStreamSynchronize(c->stream) != cudaSuccess && !r) r = CLIFFS_ERR_CUDA;
  cudaFree(buf);
  return r ? r : 1;
}

// ---------------------------------------------------------------------------
// Asynchronous outputs.

namespace {

// The next output slot, with a device buffer of at least `bytes`.  The
// context's stream first waits until the slot's previous copy has left it.
int out_slot(cliffs_ctx* c, size_t bytes, OutSlot** slot, int64_t* ticket) {
  if (!c->cpy) {
    CK(cudaStreamCreateWithFlags(&c->cpy, cudaStreamNonBlocking));
    for (auto& o : c->outs) {
      CK(cudaEventCreateWithFlags(&o.conv, cudaEventDisableTiming));
      CK(cudaEventCreateWithFlags(&o.done, cudaEventDisableTiming));
    }
  }
  OutSlot& o = c->outs[c->out_next % kOutSlots];
  if (o.cap < bytes) {
    if (o.used) CK(cudaEventSynchronize(o.done));
    if (o.dbuf) cudaFree(o.dbuf);
    o.dbuf = nullptr;
    o.cap = 0;
    if (cudaMalloc(&o.dbuf, bytes) != cudaSuccess) return CLIFFS_ERR_NOMEM;
    o.cap = bytes;
  } else if (o.used) {
    CK(cudaStreamWaitEvent(c->stream, o.done, 0));
  }
  o.used = true;
  *slot = &o;
  *ticket = c->out_next++;
  return CLIFFS_OK;
}

struct HostCopy {
  void* dst;
  const void* src;
  size_t bytes;
};

// After the conversion kernels on the context's stream: the copies to the
// host, on the copy stream behind them.
int out_copy(cliffs_ctx* c, OutSlot& o, std::initializer_list<HostCopy> copies) {
  CK(cudaEventRecord(o.conv, c->stream));
  CK(cudaStreamWaitEvent(c->cpy, o.conv, 0));
  for (const HostCopy& h : copies)
    if (h.bytes) CK(cudaMemcpyAsync(h.dst, h.src, h.bytes, cudaMemcpyDeviceToHost, c->cpy));
  CK(cudaEventRecord(o.done, c->cpy));
  return CLIFFS_OK;
}

}  // namespace

int cliffs_gpu_get_sea_state_async(cliffs_ctx* c, int32_t lonsub, int32_t latsub, float* h, float* u, float* v,
                                   int64_t* ticket) {
  if (!c || lonsub < 1 || latsub < 1 || !h || !u || !v || !ticket) return CLIFFS_ERR_ARG;
  if (!c->have_state) return CLIFFS_ERR_STATE;
  const int nxs = (c->nx - 1) / lonsub + 1, nys = (c->ny - 1) / latsub + 1;
  const size_t n = (size_t)nxs * nys;
  OutSlot* o = nullptr;
  int64_t tk = 0;
  int r = out_slot(c, 3 * n * sizeof(float), &o, &tk);
  if (r) return r;
  float* a = (float*)o->dbuf;
  const int s = c->cur;
  ++c->launches;
  k_sea_state<<<grid2(nxs, nys), 128, 0, c->stream>>>(nxs, nys, c->pitch, lonsub, latsub, c->dep, c->srf[s],
                                                      c->xu[s], c->yv[s], (float)c->ground, a, a + n, a + 2 * n);
  CK(cudaGetLastError());
  r = out_copy(c, *o, {{h, a, n * 4}, {u, a + n, n * 4}, {v, a + 2 * n, n * 4}});
  if (r) return r;
  *ticket = tk;
  return CLIFFS_OK;
}

int cliffs_gpu_get_gauges_async(cliffs_ctx* c, int32_t n, const int32_t* I, const int32_t* J, double* eta,
                                double* u, double* v, int64_t* ticket) {
  if (!c || n < 1 || !I || !J || !eta || !u || !v || !ticket) return CLIFFS_ERR_ARG;
  if (!c->have_state) return CLIFFS_ERR_STATE;
  for (int k = 0; k < n; ++k)
    if (I[k] < 1 || I[k] > c->nx || J[k] < 1 || J[k] > c->ny) return CLIFFS_ERR_ARG;
  // the indices stay on the device; a new set goes up (synchronously) once
  const bool same = n == c->g_n && std::equal(I, I + n, c->g_host.begin()) &&
                    std::equal(J, J + n, c->g_host.begin() + n);
  if (!same) {
    CK(cudaStreamSynchronize(c->stream));
    if (c->g_cap < n) {
      if (c->g_ij) cudaFree(c->g_ij);
      c->g_ij = nullptr;
      c->g_cap = 0;
      if (dalloc(&c->g_ij, 2 * (size_t)n)) return CLIFFS_ERR_NOMEM;
      c->g_cap = n;
    }
    c->g_host.assign(I, I + n);
    c->g_host.insert(c->g_host.end(), J, J + n);
    CK(cudaMemcpy(c->g_ij, c->g_host.data(), 2 * (size_t)n * 4, cudaMemcpyHostToDevice));
    c->g_n = n;
  }
  OutSlot* o = nullptr;
  int64_t tk = 0;
  int r = out_slot(c, 3 * (size_t)n * sizeof(double), &o, &tk);
  if (r) return r;
  double* out = (double*)o->dbuf;
  const int s = c->cur;
  ++c->launches;
  k_gauges<<<(n + 127) / 128, 128, 0, c->stream>>>(n, c->g_ij, c->g_ij + n, c->pitch, c->dep, c->srf[s], c->xu[s],
                                                   c->yv[s], (float)c->ground, out);
  CK(cudaGetLastError());
  r = out_copy(c, *o, {{eta, out, (size_t)n * 8}, {u, out + n, (size_t)n * 8}, {v, out + 2 * n, (size_t)n * 8}});
  if (r) return r;
  *ticket = tk;
  return CLIFFS_OK;
}

int cliffs_gpu_feed_child_async(cliffs_ctx* c, int32_t id, double cuke, int32_t* arrived, double* w, double* e,
                                double* s, double* nn_out, int64_t* ticket) {
  if (!c || !arrived || !w || !e || !s || !nn_out || !ticket || id < 0 || id >= (int32_t)c->nests.size())
    return CLIFFS_ERR_ARG;
  if (!c->have_state) return CLIFFS_ERR_STATE;
  const Nest& n = c->nests[id];
  const int mm = n.d.mm, nn = n.d.nn;
  const size_t rec = 6 * (size_t)(mm + nn);
  OutSlot* o = nullptr;
  int64_t tk = 0;
  int r = out_slot(c, rec * sizeof(double) + sizeof(double), &o, &tk);
  if (r) return r;
  double* buf = (double*)o->dbuf;
  double *dw = buf, *de = buf + 3 * (size_t)nn, *ds = buf + 6 * (size_t)nn, *dn = ds + 3 * (size_t)mm;
  int* gate = (int*)(buf + rec);
  const int st = c->cur;
  c->launches += 2;
  // the arrival test leaves at once when an earlier call found the wave
  k_arrival<<<152, 256, 0, c->stream>>>(n.i1, n.i2, n.k1, n.k2, c->pitch, c->dep, c->srf[st], c->xu[st],
                                        c->yv[st], c->ground, cuke, kGrav, n.d_arr, true);
  CK(cudaGetLastError());
  const int threads = 2 * (mm + nn);
  k_feed_child<<<(threads + 127) / 128, 128, 0, c->stream>>>(
      mm, nn, n.d.W_nx, n.d.E_nx, n.d.S_ny, n.d.N_ny, n.d.W_cx, n.d.E_cx, n.d.S_cy, n.d.N_cy, n.WE_ny, n.WE_cy,
      n.SN_nx, n.SN_cx, c->pitch, c->dep, c->srf[st], c->xu[st], c->yv[st], c->ground, kGrav, dw, de, ds, dn,
      n.d_arr, gate);
  CK(cudaGetLastError());
  r = out_copy(c, *o,
               {{w, dw, 3 * (size_t)nn * 8}, {e, de, 3 * (size_t)nn * 8}, {s, ds, 3 * (size_t)mm * 8},
                {nn_out, dn, 3 * (size_t)mm * 8}, {arrived, gate, sizeof(int32_t)}});
  if (r) return r;
  *ticket = tk;
  return CLIFFS_OK;
}

int cliffs_gpu_output_wait(cliffs_ctx* c, int64_t ticket) {
  if (!c || ticket < 0 || ticket >= c->out_next) return CLIFFS_ERR_ARG;
  // a later output of the same slot follows this one on the copy stream
  CK(cudaEventSynchronize(c->outs[ticket % kOutSlots].done));
  return CLIFFS_OK;
}

int cliffs_gpu_output_done(cliffs_ctx* c, int64_t ticket, int32_t* done) {
  if (!c || !done || ticket < 0 || ticket >= c->out_next) return CLIFFS_ERR_ARG;
  const cudaError_t q = cudaEventQuery(c->outs[ticket % kOutSlots].done);
  if (q != cudaSuccess && q != cudaErrorNotReady) return CLIFFS_ERR_CUDA;
  *done = q == cudaSuccess ? 1 : 0;
  return CLIFFS_OK;
}

int cliffs_gpu_host_alloc(int64_t bytes, void** p) {
  if (!p || bytes < 1) return CLIFFS_ERR_ARG;
  return cudaHostAlloc(p, (size_t)bytes, cudaHostAllocDefault) == cudaSuccess ? CLIFFS_OK : CLIFFS_ERR_NOMEM;
}

void cliffs_gpu_host_free(void* p) {
  if (p) cudaFreeHost(p);
}

int cliffs_gpu_status(cliffs_ctx* c, uint32_t* flags) {
  if (!c || !flags) return CLIFFS_ERR_ARG;
  unsigned w[2] = {0, 0};
  CK(cudaMemcpyAsync(w, c->status, sizeof(w), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaMemsetAsync(c->status, 0, sizeof(w), c->stream));
  CK(cudaStreamSynchronize(c->stream));
  *flags = w[0];
  float courant = 0.f;
  std::memcpy(&courant, &w[1], sizeof(float));
  c->courant_seen = std::max(c->courant_seen, (double)courant);
  if (w[0] & CLIFFS_ST_NAN) return CLIFFS_ERR_NAN;
  if (w[0] & CLIFFS_ST_STALL) return CLIFFS_ERR_TIMEOUT;
  return (w[0] & CLIFFS_ST_CFL) ? CLIFFS_WARN_CFL : CLIFFS_OK;
}

int cliffs_gpu_courant(cliffs_ctx* c, double* courant) {
  if (!c || !courant) return CLIFFS_ERR_ARG;
  unsigned w[2] = {0, 0};
  CK(cudaMemcpyAsync(w, c->status, sizeof(w), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  float now = 0.f;
  std::memcpy(&now, &w[1], sizeof(float));
  *courant = std::max(c->courant_seen, (double)now);
  return CLIFFS_OK;
}

int cliffs_gpu_set_sweep_kernel(cliffs_ctx* c, int32_t kind) {
  if (!c || (kind != CLIFFS_SWEEP_TILED && kind != CLIFFS_SWEEP_STAGED && kind != CLIFFS_SWEEP_DIRECT))
    return CLIFFS_ERR_ARG;
  if (c->have_state) RET(max_sync(c));  // the staged kernels fold nothing in
  c->sweep_kind = kind;
  return CLIFFS_OK;
}

int cliffs_gpu_check_stage_timeout(cliffs_ctx* c, int32_t wait_ms) {
  if (!c || wait_ms < 1 || wait_ms > 2000) return CLIFFS_ERR_ARG;
  if (!c->have_state || !c->staged_ok || !c->xrun) return CLIFFS_ERR_STATE;
  const SweepArgs A = sweep_args(c, 1, false, c->cur);  // writes copy 1 - cur, which stays unused
  const StageCtl S{(unsigned long long)wait_ms * 1000000ull, 16u};
  const int tiles = (A.n + kXTile - 1) / kXTile * A.nlines;
  ++c->launches;
  staged_x<<<std::min(tiles, c->grid_sx), kStagedThreads, 0, c->stream>>>(A, S);
  CK(cudaGetLastError());
  unsigned f = 0;
  CK(cudaMemcpyAsync(&f, c->status, sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaMemsetAsync(c->status, 0, sizeof(unsigned), c->stream));
  CK(cudaStreamSynchronize(c->stream));
  if (!(f & ST_STALL)) return CLIFFS_OK;
  if (c->yrun && c->ytile_ok) {
    // the same for one tiled y-sweep (tile_y_kernel): its copy waits run out
    const SweepArgs Ay = sweep_args(c, 2, false, c->cur);  // writes copy 1 - cur too
    const int s = c->cur;
    const YTileMaps M{c->m_dep, c->m_srf[s], c->m_xu[s], c->m_yv[s], c->m_srf16[1 - s], c->m_xu16[1 - s],
                      c->m_yv16[1 - s]};
    const dim3 grid((Ay.nlines + 31) / 32, (Ay.n + kYRows - 1) / kYRows);
    ++c->launches;
    if (Ay.geo_uniform && Ay.scl == nullptr)
      tile_y_kernel<true><<<grid, kStagedThreads, 0, c->stream>>>(Ay, M, S);
    else
      tile_y_kernel<false><<<grid, kStagedThreads, 0, c->stream>>>(Ay, M, S);
    CK(cudaGetLastError());
    f = 0;
    CK(cudaMemcpyAsync(&f, c->status, sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemsetAsync(c->status, 0, sizeof(unsigned), c->stream));
    CK(cudaStreamSynchronize(c->stream));
  }
  return (f & ST_STALL) ? CLIFFS_ERR_TIMEOUT : CLIFFS_OK;
}

int cliffs_gpu_sync(cliffs_ctx* c) {
  if (!c) return CLIFFS_ERR_ARG;
  CK(cudaStreamSynchronize(c->stream));
  return CLIFFS_OK;
}

int cliffs_gpu_profile(cliffs_ctx* c, int32_t enable) {
  if (!c) return CLIFFS_ERR_ARG;
  int r = flush_profile(c);
  c->prof = enable != 0;
  c->prof_ms[0] = c->prof_ms[1] = 0;
  c->prof_n[0] = c->prof_n[1] = 0;
  return r;
}

int cliffs_gpu_profile_read(cliffs_ctx* c, double* x_ms, int64_t* x_n, double* y_ms, int64_t* y_n) {
  if (!c) return CLIFFS_ERR_ARG;
  int r = flush_profile(c);
  if (r) return r;
  if (x_ms) *x_ms = c->prof_n[0] ? c->prof_ms[0] / c->prof_n[0] : 0.0;
  if (x_n) *x_n = c->prof_n[0];
  if (y_ms) *y_ms = c->prof_n[1] ? c->prof_ms[1] / c->prof_n[1] : 0.0;
  if (y_n) *y_n = c->prof_n[1];
  return CLIFFS_OK;
}

int cliffs_gpu_launch_count(cliffs_ctx* c, int64_t* n) {
  if (!c || !n) return CLIFFS_ERR_ARG;
  *n = c->launches;
  return CLIFFS_OK;
}

int cliffs_gpu_set_tiling(cliffs_ctx* c, int32_t block_x, int32_t warps_y) {
  if (!c || block_x < 0 || warps_y < 0 || block_x % 32 || block_x > 256 || warps_y > 8) return CLIFFS_ERR_ARG;
  if (block_x) c->blk_x = block_x;
  if (warps_y) c->warps_y = warps_y;
  return CLIFFS_OK;
}

// ---------------------------------------------------------------------------
// Sweep without device allocation.
//
// Callers that cannot allocate device memory use this entry point, e.g. a host
// application that hands the solver a fixed memory budget up front and
// forbids cudaMalloc afterwards, or a time loop that must not pay
// cudaMalloc's implicit device synchronisation on every call.  The sweep's
// only scratch, the worklist of cells that need the full wet/dry rules (and
// its counters), lives in the fixed-size arrays below instead of memory the
// library allocates.  Every GPU that loads this library holds them until the
// process exits: kNoAllocCells * 4 bytes plus a few words.
// ---------------------------------------------------------------------------

static constexpr int kNoAllocCells = 1 << 20;  // largest nx*ny accepted
static __device__ __align__(256) uint32_t g_noalloc_list[kNoAllocCells];
// [0] worklist length of the current call (afterwards: the cells it listed),
// [1] the other parity's counter (zeroed by the fast kernel), [2] status bits,
// [3] the largest Courant number above 1 (float bits)
static __device__ __align__(256) uint32_t g_noalloc_words[4];

struct NoAllocScratch {
  uint32_t* list = nullptr;
  uint32_t* words = nullptr;
};

// Device addresses of the scratch arrays, resolved once per device with that
// device current.  In host code the array names are host-side stand-ins, never
// device addresses.  Host threads making their first calls at the same time
// serialise on the lock; later calls read the published entry without it.
static int noalloc_scratch(NoAllocScratch* out) {
  constexpr int kMaxDevices = 64;
  static NoAllocScratch cache[kMaxDevices];
  static std::atomic<bool> ready[kMaxDevices];
  static std::mutex lock;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return CLIFFS_ERR_DEVICE;
  if (!ready[dev].load(std::memory_order_acquire)) {
    std::lock_guard<std::mutex> g(lock);
    if (!ready[dev].load(std::memory_order_relaxed)) {
      void *a = nullptr, *b = nullptr;
      if (cudaGetSymbolAddress(&a, g_noalloc_list) != cudaSuccess ||
          cudaGetSymbolAddress(&b, g_noalloc_words) != cudaSuccess)
        return CLIFFS_ERR_CUDA;
      cache[dev].list = (uint32_t*)a;
      cache[dev].words = (uint32_t*)b;
      ready[dev].store(true, std::memory_order_release);
    }
  }
  *out = cache[dev];
  return CLIFFS_OK;
}

int cliffs_gpu_sweep_noalloc(int32_t iu, int32_t nx, int32_t ny, int32_t pitch, const float* dep,
                             const float* srf, const float* xvel, const float* yvel, float* srf_out,
                             float* xvel_out, float* yvel_out, double dx, double dy, double ground,
                             double crough, double dt, void* stream) {
  if (iu != 1 && iu != 2) return CLIFFS_ERR_ARG;
  if (nx < 1 || ny < 1 || (nx <= 2 && ny <= 2)) return CLIFFS_ERR_ARG;
  if ((iu == 1 && nx <= 2) || (iu == 2 && ny <= 2)) return CLIFFS_ERR_ARG;
  if ((int64_t)nx * (int64_t)ny > kNoAllocCells) return CLIFFS_ERR_ARG;
  if (pitch < nx || pitch % 4 != 0) return CLIFFS_ERR_ARG;
  const void* ptrs[] = {dep, srf, xvel, yvel, srf_out, xvel_out, yvel_out};
  for (const void* q : ptrs)
    if (!q || ((uintptr_t)q % 16) != 0) return CLIFFS_ERR_ARG;
  if (!(dt > 0) || !(ground > 0) || crough < 0) return CLIFFS_ERR_ARG;
  if ((iu == 1 && !(dx > 0)) || (iu == 2 && !(dy > 0))) return CLIFFS_ERR_ARG;
  NoAllocScratch sc;
  int r = noalloc_scratch(&sc);
  if (r) return r;
  cudaStream_t st = (cudaStream_t)stream;
  SweepArgs A{};
  A.pitch = pitch;
  A.dep = dep;
  A.srf = srf;
  A.xu = xvel;
  A.yv = yvel;
  A.srf_o = srf_out;
  A.xu_o = xvel_out;
  A.yv_o = yvel_out;
  A.hmax = nullptr;
  A.velmax = nullptr;
  A.ph.g = (float)kGrav;
  A.ph.ginv = (float)(1.0 / kGrav);
  A.ph.ground = (float)ground;
  A.ph.celmin = (float)sqrt(kGrav * ground);
  A.ph.dt = (float)dt;
  A.ph.idt = (float)(1.0 / dt);
  A.ph.gcrough = (float)(kGrav * crough);
  A.ph.sqr2 = (float)kSqr2;
  const double h = iu == 1 ? dx : dy;  // uniform spacing along the line
  A.geo = nullptr;
  A.geo_uniform = 1;
  A.geo0 = make_float4((float)(1.0 / h), (float)(1.0 / h), (float)(dt / (2.0 * h)), 0.f);
  A.scl = nullptr;
  A.lscale = nullptr;
  A.inv_dx1 = A.inv_dxn1 = (float)(1.0 / h);
  A.edges = nullptr;
  A.list = sc.list;
  A.count = sc.words;
  A.count_next = sc.words + 1;
  A.status = (unsigned*)(sc.words + 2);
  // the shared words keep the previous call's values: the counter, the
  // status and the Courant word start from zero
  CK(cudaMemsetAsync(sc.words, 0, 4 * sizeof(uint32_t), st));
  if (iu == 1) {
    A.n = nx;
    A.nlines = ny;
    A.lo = ny > 2 ? 2 : 1;
    A.hi = ny > 2 ? ny - 1 : 1;
    const dim3 grid((nx + 128 * kCellsPerThread - 1) / (128 * kCellsPerThread), ny);
    fast_kernel<0, false><<<grid, 128, 0, st>>>(A);
    CK(cudaGetLastError());
    general_kernel<0><<<kGeneralBlocks, 128, 0, st>>>(A);
  } else {
    A.n = ny;
    A.nlines = nx;
    A.lo = nx > 2 ? 2 : 1;
    A.hi = nx > 2 ? nx - 1 : 1;
    const dim3 grid((ny + 8 * kCellsPerThread - 1) / (8 * kCellsPerThread), (nx + 31) / 32);
    fast_kernel<1, false><<<grid, 256, 0, st>>>(A);
    CK(cudaGetLastError());
    general_kernel<1><<<kGeneralBlocks, 128, 0, st>>>(A);
  }
  CK(cudaGetLastError());
  return CLIFFS_OK;
}

int cliffs_gpu_sweep_noalloc_status(void* stream, uint32_t* flags, uint32_t* listed) {
  NoAllocScratch sc;
  int r = noalloc_scratch(&sc);
  if (r) return r;
  cudaStream_t st = (cudaStream_t)stream;
  uint32_t w[4] = {0, 0, 0, 0};
  CK(cudaMemcpyAsync(w, sc.words, sizeof(w), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  if (flags) *flags = w[2];
  if (listed) *listed = w[0];
  return (w[2] & ST_NAN) ? CLIFFS_ERR_NAN : CLIFFS_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Ensembles: many contexts stepped together (batch.cuh).
// ---------------------------------------------------------------------------

struct cliffs_batch {
  std::vector<cliffs_ctx*> ctx;
  int dev = 0, sms = 0, max_ctas = 0;
  cudaStream_t stream = nullptr;
  SweepArgs* d_args = nullptr;       // fused set
  SweepArgs* d_args_fold = nullptr;  // fold set
  int* d_off = nullptr;
  int* d_gx = nullptr;
  unsigned* d_sync = nullptr;  // [0] barrier counter, [1] timeout flag
  int total[2] = {0, 0};
  // every scenario flat along x / y (uniform spacing, no metric term): the
  // one-tile phases run their flat variant
  bool flat[2] = {false, false};
  // every scenario's tensor maps made: the one-tile y phase of the fold set
  // runs batch_tile_y when flat along y
  YTileMaps* d_ymaps = nullptr;
  bool ytile = false;
  // per scenario, in single-grid tiles: x (column chunks, rows), y (row
  // groups, column groups); the list of a plan's tile shape is built from them
  std::vector<int> tx, ty, lx, ly;
  cliffs_batch_plan plan{CLIFFS_BATCH_PERSISTENT, 1, 32, 1, 1};
  // gauges of every scenario (cliffs_batch_set_gauges): scenario, I, J per
  // entry, and the device record of (eta, u, v)
  int32_t* d_gauge = nullptr;
  double* d_grec = nullptr;
  int gauges = 0;
  // [0]: graph of plan.graph_steps steps; [1]: the last steps of a call,
  // when fewer (at least 2)
  cudaGraphExec_t graph[2] = {nullptr, nullptr};
  int graph_built[2] = {0, 0};  // steps in each instantiated graph
  int64_t launches = 0;
};

static BatchArgs batch_args(const cliffs_batch* b, int steps, bool fold) {
  BatchArgs B;
  B.args = fold ? b->d_args_fold : b->d_args;
  B.off = b->d_off;
  B.gx = b->d_gx;
  B.n = (int)b->ctx.size();
  B.steps = steps;
  B.bar = b->d_sync;
  B.err = b->d_sync + 1;
  B.wait_ns = kBarrierNs;
  B.extra = 0;
  B.span[0] = std::max(1, b->plan.x_rows);
  B.span[1] = std::max(1, b->plan.y_groups);
  B.ymaps = b->d_ymaps;
  return B;
}

// The tile lists of the plan's tile shape: per direction, the offset of each
// scenario's first list entry and its entries along the first tile dimension.
static int batch_lists(cliffs_batch* b) {
  const int n = (int)b->ctx.size();
  const int sx = std::max(1, b->plan.x_rows), sy = std::max(1, b->plan.y_groups);
  std::vector<int> off(2 * ((size_t)n + 1), 0), gx(2 * (size_t)n, 0);
  for (int k = 0; k < n; ++k) {
    gx[k] = b->tx[k];                        // column chunks
    gx[n + k] = (b->ty[k] + sy - 1) / sy;    // entries of sy row groups
    off[k + 1] = off[k] + gx[k] * ((b->lx[k] + sx - 1) / sx);
    off[(n + 1) + k + 1] = off[(n + 1) + k] + gx[n + k] * b->ly[k];
  }
  b->total[0] = off[n];
  b->total[1] = off[(n + 1) + n];
  if (cudaMemcpy(b->d_off, off.data(), off.size() * sizeof(int), cudaMemcpyHostToDevice) ||
      cudaMemcpy(b->d_gx, gx.data(), gx.size() * sizeof(int), cudaMemcpyHostToDevice))
    return CLIFFS_ERR_CUDA;
  return CLIFFS_OK;
}

static void batch_free(cliffs_batch* b) {
  for (cudaGraphExec_t g : b->graph)
    if (g) cudaGraphExecDestroy(g);
  if (b->d_args) cudaFree(b->d_args);
  if (b->d_args_fold) cudaFree(b->d_args_fold);
  if (b->d_off) cudaFree(b->d_off);
  if (b->d_gx) cudaFree(b->d_gx);
  if (b->d_sync) cudaFree(b->d_sync);
  if (b->d_gauge) cudaFree(b->d_gauge);
  if (b->d_grec) cudaFree(b->d_grec);
  if (b->d_ymaps) cudaFree(b->d_ymaps);
  if (b->stream) cudaStreamDestroy(b->stream);
}

int cliffs_batch_create(cliffs_ctx* const* ctxs, int32_t n, cliffs_batch** out) {
  if (!ctxs || n < 1 || !out) return CLIFFS_ERR_ARG;
  *out = nullptr;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return CLIFFS_ERR_DEVICE;
  for (int k = 0; k < n; ++k) {
    const cliffs_ctx* c = ctxs[k];
    if (!c || c->dev != dev || !c->xrun || !c->yrun || c->feed_on || c->edges_static) return CLIFFS_ERR_ARG;
    if (!c->have_state) return CLIFFS_ERR_STATE;
  }
  int coop = 0;
  cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
  auto* b = new cliffs_batch;
  b->ctx.assign(ctxs, ctxs + n);
  b->dev = dev;
  auto fail = [&](int r) {
    batch_free(b);
    delete b;
    return r;
  };
  if (cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return fail(CLIFFS_ERR_CUDA);
  int ctas_fold = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b->max_ctas, batch_persistent<true>, kBatchThreads, 0) !=
          cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&ctas_fold, batch_persistent<false>, kBatchThreads, 0) !=
          cudaSuccess)
    return fail(CLIFFS_ERR_CUDA);
  b->max_ctas = std::min(b->max_ctas, ctas_fold);  // resident with either argument set
  if (!coop) b->max_ctas = 0;  // graph schedule only
  // per scenario: the x-sweep reads copy cur and writes 1-cur, the y-sweep
  // reads 1-cur and writes cur; the max-wave update in the y-sweep (fused
  // set) or the previous end state folded in by the x-sweep (fold set)
  std::vector<SweepArgs> args(2 * (size_t)n), fold(2 * (size_t)n);
  std::vector<int> off(2 * ((size_t)n + 1), 0), gx(2 * (size_t)n, 0);
  b->flat[0] = b->flat[1] = true;
  for (int k = 0; k < n; ++k) {
    cliffs_ctx* c = ctxs[k];
    b->flat[0] = b->flat[0] && c->geo_uni_x;  // the x-sweep has no metric term
    b->flat[1] = b->flat[1] && c->geo_uni_y && c->scl_y == nullptr;
    if (cudaStreamSynchronize(c->stream) != cudaSuccess) return fail(CLIFFS_ERR_CUDA);
    args[2 * k] = sweep_args(c, 1, false, c->cur);
    args[2 * k + 1] = sweep_args(c, 2, true, 1 - c->cur);
    fold[2 * k] = args[2 * k];
    fold[2 * k].hmax_in = c->hmax;
    fold[2 * k].velmax_in = c->velmax;
    fold[2 * k + 1] = sweep_args(c, 2, false, 1 - c->cur);
    b->tx.push_back((c->nx + kBatchThreads * kCellsPerThread - 1) / (kBatchThreads * kCellsPerThread));
    b->lx.push_back(c->ny);
    b->ty.push_back((c->ny + (kBatchThreads / 32) * kCellsPerThread - 1) / ((kBatchThreads / 32) * kCellsPerThread));
    b->ly.push_back((c->nx + 31) / 32);
  }
  if (dalloc(&b->d_args, args.size()) || dalloc(&b->d_args_fold, fold.size()) || dalloc(&b->d_off, off.size()) ||
      dalloc(&b->d_gx, gx.size()) || dalloc(&b->d_sync, 2))
    return fail(CLIFFS_ERR_NOMEM);
  if (cudaMemcpy(b->d_args, args.data(), args.size() * sizeof(SweepArgs), cudaMemcpyHostToDevice) ||
      cudaMemcpy(b->d_args_fold, fold.data(), fold.size() * sizeof(SweepArgs), cudaMemcpyHostToDevice) ||
      batch_lists(b) || cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking))
    return fail(CLIFFS_ERR_CUDA);
  {
    // the y-sweep of scenario k reads state copy 1 - cur and writes cur
    std::vector<YTileMaps> ym((size_t)n);
    bool ok = true;
    for (int k = 0; k < n && ok; ++k) {
      const cliffs_ctx* c = ctxs[k];
      ok = c->ytile_ok;
      const int s = 1 - c->cur;
      if (ok)
        ym[k] = YTileMaps{c->m_dep, c->m_srf[s], c->m_xu[s], c->m_yv[s], c->m_srf16[c->cur], c->m_xu16[c->cur],
                          c->m_yv16[c->cur]};
    }
    if (ok && b->flat[1]) {
      if (dalloc(&b->d_ymaps, ym.size())) return fail(CLIFFS_ERR_NOMEM);
      if (cudaMemcpy(b->d_ymaps, ym.data(), ym.size() * sizeof(YTileMaps), cudaMemcpyHostToDevice))
        return fail(CLIFFS_ERR_CUDA);
      b->ytile = true;
    }
  }
  b->plan.mode = b->max_ctas > 0 ? CLIFFS_BATCH_PERSISTENT : CLIFFS_BATCH_GRAPH;
  b->plan.ctas_per_sm = std::max(1, b->max_ctas);
  b->plan.graph_steps = 32;
  *out = b;
  return CLIFFS_OK;
}

void cliffs_batch_destroy(cliffs_batch* b) {
  if (!b) return;
  if (b->stream) cudaStreamSynchronize(b->stream);
  batch_free(b);
  delete b;
}

int cliffs_batch_set_plan(cliffs_batch* b, const cliffs_batch_plan* p) {
  if (!b || !p) return CLIFFS_ERR_ARG;
  if (p->mode == CLIFFS_BATCH_PERSISTENT) {
    if (p->ctas_per_sm < 1 || p->ctas_per_sm > b->max_ctas) return CLIFFS_ERR_ARG;
  } else if (p->mode == CLIFFS_BATCH_GRAPH) {
    if (p->graph_steps < 1 || p->graph_steps > 4096) return CLIFFS_ERR_ARG;
  } else {
    return CLIFFS_ERR_ARG;
  }
  if (p->x_rows < 0 || p->x_rows > 64 || p->y_groups < 0 || p->y_groups > 64) return CLIFFS_ERR_ARG;
  const bool shape = std::max(1, p->x_rows) != std::max(1, b->plan.x_rows) ||
                     std::max(1, p->y_groups) != std::max(1, b->plan.y_groups);
  b->plan = *p;
  b->plan.x_rows = std::max(1, p->x_rows);
  b->plan.y_groups = std::max(1, p->y_groups);
  if (shape) {
    // the captured graphs hold the old list sizes
    for (int s = 0; s < 2; ++s) {
      if (b->graph[s]) cudaGraphExecDestroy(b->graph[s]);
      b->graph[s] = nullptr;
      b->graph_built[s] = 0;
    }
    CK(cudaStreamSynchronize(b->stream));
    RET(batch_lists(b));
  }
  return CLIFFS_OK;
}

int cliffs_batch_get_plan(const cliffs_batch* b, cliffs_batch_plan* p) {
  if (!b || !p) return CLIFFS_ERR_ARG;
  *p = b->plan;
  return CLIFFS_OK;
}

int cliffs_batch_launch_count(const cliffs_batch* b, int64_t* n) {
  if (!b || !n) return CLIFFS_ERR_ARG;
  *n = b->launches;
  return CLIFFS_OK;
}

static int batch_launch_phases(cliffs_batch* b, int steps, bool fold) {
  const BatchArgs B = batch_args(b, 1, fold);
  const bool mx = B.span[0] > 1, my = B.span[1] > 1;
  const bool fx = b->flat[0], fy = b->flat[1];
  for (int s = 0; s < steps; ++s) {
    if (mx)
      batch_phase<0, false, true><<<b->total[0], kBatchThreads, 0, b->stream>>>(B);
    else if (fx)
      batch_phase<0, false, false, true><<<b->total[0], kBatchThreads, 0, b->stream>>>(B);
    else
      batch_phase<0, false, false><<<b->total[0], kBatchThreads, 0, b->stream>>>(B);
    if (fold) {
      if (my)
        batch_phase<1, false, true><<<b->total[1], kBatchThreads, 0, b->stream>>>(B);
      else if (fy && b->ytile)
        batch_tile_y<true><<<b->total[1], kBatchThreads, 0, b->stream>>>(B);
      else if (fy)
        batch_phase<1, false, false, true><<<b->total[1], kBatchThreads, 0, b->stream>>>(B);
      else
        batch_phase<1, false, false><<<b->total[1], kBatchThreads, 0, b->stream>>>(B);
    } else {
      if (my)
        batch_phase<1, true, true><<<b->total[1], kBatchThreads, 0, b->stream>>>(B);
      else if (fy)
        batch_phase<1, true, false, true><<<b->total[1], kBatchThreads, 0, b->stream>>>(B);
      else
        batch_phase<1, true, false><<<b->total[1], kBatchThreads, 0, b->stream>>>(B);
    }
    b->launches += 2;
  }
  return cudaGetLastError() == cudaSuccess ? CLIFFS_OK : CLIFFS_ERR_CUDA;
}

static int batch_build_graph(cliffs_batch* b, int slot, int steps) {
  if (b->graph[slot]) {
    cudaGraphExecDestroy(b->graph[slot]);
    b->graph[slot] = nullptr;
    b->graph_built[slot] = 0;
  }
  const int64_t before = b->launches;
  cudaGraph_t g = nullptr;
  CK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
  const int r = batch_launch_phases(b, steps, true);
  const cudaError_t e = cudaStreamEndCapture(b->stream, &g);
  b->launches = before;  // captured, not launched
  if (r || e != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    return CLIFFS_ERR_CUDA;
  }
  const cudaError_t ie = cudaGraphInstantiate(&b->graph[slot], g, 0);
  cudaGraphDestroy(g);
  if (ie != cudaSuccess) {
    b->graph[slot] = nullptr;
    return CLIFFS_ERR_CUDA;
  }
  b->graph_built[slot] = steps;
  return CLIFFS_OK;
}

// Steps while a source is still rising: each rising context's share of the
// step (as cliffs_gpu_step applies it), then the batched sweep phases.
static int batch_rising_steps(cliffs_batch* b, int* nsteps) {
  int r = CLIFFS_OK;
  auto rising = [&]() {
    for (cliffs_ctx* c : b->ctx)
      if (c->rise_on) return true;
    return false;
  };
  while (*nsteps > 0 && !r && rising()) {
    for (cliffs_ctx* c : b->ctx) {
      if (!c->rise_on) continue;
      c->rise_el += c->dt;
      const double w = std::min(1.0, c->rise_el / c->rise_T);
      k_add_surface<<<grid2(c->nx, c->ny), 128, 0, b->stream>>>(c->nx, c->ny, c->pitch, c->dep, c->srf[c->cur],
                                                                 c->rise_q, (float)w, (float)c->rise_w,
                                                                 (float)c->ground);
      ++b->launches;
      c->rise_w = w;
      if (w >= 1.0) c->rise_on = false;
    }
    r = batch_launch_phases(b, 1, false);
    for (cliffs_ctx* c : b->ctx) c->sweeps += 2u;
    --*nsteps;
  }
  if (cudaStreamSynchronize(b->stream) != cudaSuccess && !r) r = CLIFFS_ERR_CUDA;
  return r;
}

int cliffs_batch_step(cliffs_batch* b, int32_t nsteps) {
  if (!b || nsteps < 0) return CLIFFS_ERR_ARG;
  if (nsteps == 0) return CLIFFS_OK;
  // Steps with the fused argument set (a fresh state's first step, the steps
  // of a rising source) fold nothing in: pending end states go in first.
  bool fused_first = false;
  for (cliffs_ctx* c : b->ctx) fused_first = fused_first || c->max_fresh || c->rise_on;
  if (fused_first)
    for (cliffs_ctx* c : b->ctx)
      if (c->max_pending) {
        RET(max_sync(c));
        CK(cudaStreamSynchronize(c->stream));
      }
  for (cliffs_ctx* c : b->ctx) c->max_fresh = false;
  const int before = nsteps;
  int r = batch_rising_steps(b, &nsteps);
  if (r) return r;
  if (fused_first && nsteps == before) {  // a fresh state's first step
    r = batch_launch_phases(b, 1, false);
    for (cliffs_ctx* c : b->ctx) c->sweeps += 2u;
    --nsteps;
    if (r) return r;
  }
  // the end state is folded in by the next x-sweep, or by max_sync
  for (cliffs_ctx* c : b->ctx) c->max_pending = nsteps > 0;
  if (nsteps == 0) {
    CK(cudaStreamSynchronize(b->stream));
    return CLIFFS_OK;
  }
  if (b->plan.mode == CLIFFS_BATCH_PERSISTENT) {
    const int grid = b->plan.ctas_per_sm * b->sms;
    // at most 2^31 / grid barrier arrivals per launch keeps the counter exact
    const int chunk = std::max(1, std::min(100000, (int)(0x7fffffffu / (2u * (unsigned)grid)) - 1));
    for (int done = 0; done < nsteps && !r; done += chunk) {
      const int steps = std::min(chunk, nsteps - done);
      BatchArgs B = batch_args(b, steps, true);
      void* kargs[] = {&B};
      if (cudaMemsetAsync(b->d_sync, 0, 2 * sizeof(unsigned), b->stream) != cudaSuccess ||
          cudaLaunchCooperativeKernel((const void*)batch_persistent<false>, dim3(grid), dim3(kBatchThreads), kargs,
                                      0, b->stream) != cudaSuccess) {
        r = CLIFFS_ERR_CUDA;
        break;
      }
      ++b->launches;
      unsigned flags[2] = {0, 0};
      if (cudaMemcpyAsync(flags, b->d_sync, sizeof(flags), cudaMemcpyDeviceToHost, b->stream) != cudaSuccess ||
          cudaStreamSynchronize(b->stream) != cudaSuccess)
        r = CLIFFS_ERR_CUDA;
      else if (flags[1])
        r = CLIFFS_ERR_TIMEOUT;
    }
  } else {
    // graph_steps steps per replay; the last steps of the call, when fewer
    // but at least 2, from a graph of their own length
    const int k = b->plan.graph_steps;
    int done = 0;
    while (!r && nsteps - done >= 2 && k >= 2) {
      const int len = std::min(k, nsteps - done);
      const int slot = len == k ? 0 : 1;
      if (b->graph_built[slot] != len) r = batch_build_graph(b, slot, len);
      if (!r && cudaGraphLaunch(b->graph[slot], b->stream) != cudaSuccess) r = CLIFFS_ERR_CUDA;
      b->launches += 2 * (int64_t)len;
      done += len;
    }
    if (!r && done < nsteps) r = batch_launch_phases(b, nsteps - done, true);
    if (cudaStreamSynchronize(b->stream) != cudaSuccess && !r) r = CLIFFS_ERR_CUDA;
  }
  if (!r)
    for (cliffs_ctx* c : b->ctx) c->sweeps += 2u * (unsigned)nsteps;
  return r;
}

// output_gages.f:18-29 for the gauges of every scenario: entry t samples
// scenario sc[t] at (I[t], J[t]) in the state its next x-sweep reads.
__global__ void k_batch_gauges(int m, const int32_t* __restrict__ sc, const int32_t* __restrict__ I,
                               const int32_t* __restrict__ J, const SweepArgs* __restrict__ args, double* out) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= m) return;
  const SweepArgs& A = args[2 * sc[t]];
  const size_t q = (size_t)(J[t] - 1) * A.pitch + (size_t)(I[t] - 1);
  const float d = A.dep[q], s = A.srf[q];
  out[t] = depth_of(s, d) > A.ph.ground ? (double)eta_of(s, d) : (double)kNan4;
  out[m + t] = A.xu[q];
  out[2 * m + t] = A.yv[q];
}

int cliffs_batch_set_gauges(cliffs_batch* b, const int32_t* counts, const int32_t* I, const int32_t* J) {
  if (!b || !counts || !I || !J) return CLIFFS_ERR_ARG;
  const int n = (int)b->ctx.size();
  std::vector<int32_t> h;
  int m = 0;
  for (int k = 0; k < n; ++k) {
    if (counts[k] < 0) return CLIFFS_ERR_ARG;
    m += counts[k];
  }
  if (m < 1) return CLIFFS_ERR_ARG;
  h.resize(3 * (size_t)m);
  for (int k = 0, t = 0; k < n; ++k)
    for (int e = 0; e < counts[k]; ++e, ++t) {
      const cliffs_ctx* c = b->ctx[k];
      if (I[t] < 1 || I[t] > c->nx || J[t] < 1 || J[t] > c->ny) return CLIFFS_ERR_ARG;
      h[t] = k;
      h[m + t] = I[t];
      h[2 * m + t] = J[t];
    }
  CK(cudaStreamSynchronize(b->stream));
  if (b->d_gauge) cudaFree(b->d_gauge);
  if (b->d_grec) cudaFree(b->d_grec);
  b->d_gauge = nullptr;
  b->d_grec = nullptr;
  b->gauges = 0;
  if (dalloc(&b->d_gauge, h.size()) || dalloc(&b->d_grec, 3 * (size_t)m)) return CLIFFS_ERR_NOMEM;
  CK(cudaMemcpy(b->d_gauge, h.data(), h.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
  b->gauges = m;
  return CLIFFS_OK;
}

int cliffs_batch_get_gauges(cliffs_batch* b, double* eta, double* u, double* v) {
  if (!b || !eta || !u || !v) return CLIFFS_ERR_ARG;
  if (b->gauges < 1) return CLIFFS_ERR_STATE;
  const int m = b->gauges;
  k_batch_gauges<<<(m + 127) / 128, 128, 0, b->stream>>>(m, b->d_gauge, b->d_gauge + m, b->d_gauge + 2 * m,
                                                         b->d_args, b->d_grec);
  CK(cudaGetLastError());
  ++b->launches;
  CK(cudaMemcpyAsync(eta, b->d_grec, m * sizeof(double), cudaMemcpyDeviceToHost, b->stream));
  CK(cudaMemcpyAsync(u, b->d_grec + m, m * sizeof(double), cudaMemcpyDeviceToHost, b->stream));
  CK(cudaMemcpyAsync(v, b->d_grec + 2 * m, m * sizeof(double), cudaMemcpyDeviceToHost, b->stream));
  CK(cudaStreamSynchronize(b->stream));
  return CLIFFS_OK;
}

int cliffs_batch_check_barrier_timeout(cliffs_batch* b, int32_t wait_ms) {
  if (!b || wait_ms < 1 || wait_ms > 2000) return CLIFFS_ERR_ARG;
  if (b->max_ctas < 1) return CLIFFS_ERR_DEVICE;
  // the fused set: its x-sweeps, the only tiles before the first barrier,
  // leave the max-wave fields alone
  BatchArgs B = batch_args(b, 1, false);
  B.wait_ns = (unsigned long long)wait_ms * 1000000ull;
  B.extra = 1;  // an arrival no block makes: the first barrier's wait runs out
  void* kargs[] = {&B};
  const int grid = b->sms;  // one block per SM
  if (cudaMemsetAsync(b->d_sync, 0, 2 * sizeof(unsigned), b->stream) != cudaSuccess ||
      cudaLaunchCooperativeKernel((const void*)batch_persistent<true>, dim3(grid), dim3(kBatchThreads), kargs, 0,
                                  b->stream) != cudaSuccess)
    return CLIFFS_ERR_CUDA;
  ++b->launches;
  unsigned flags[2] = {0, 0};
  if (cudaMemcpyAsync(flags, b->d_sync, sizeof(flags), cudaMemcpyDeviceToHost, b->stream) != cudaSuccess ||
      cudaStreamSynchronize(b->stream) != cudaSuccess)
    return CLIFFS_ERR_CUDA;
  if (!flags[1]) return CLIFFS_OK;
  if (b->ytile) {
    // the copy waits of the batched y tiles: each expects 16 bytes more than
    // its copies bring (B.extra), runs out, and the block leaves
    BatchArgs By = batch_args(b, 1, true);
    By.wait_ns = B.wait_ns;
    By.extra = 1;
    flags[1] = 0;
    if (cudaMemsetAsync(b->d_sync, 0, 2 * sizeof(unsigned), b->stream) != cudaSuccess) return CLIFFS_ERR_CUDA;
    batch_tile_y<true><<<b->total[1], kBatchThreads, 0, b->stream>>>(By);
    ++b->launches;
    if (cudaGetLastError() != cudaSuccess ||
        cudaMemcpyAsync(flags, b->d_sync, sizeof(flags), cudaMemcpyDeviceToHost, b->stream) != cudaSuccess ||
        cudaMemsetAsync(b->d_sync, 0, 2 * sizeof(unsigned), b->stream) != cudaSuccess ||
        cudaStreamSynchronize(b->stream) != cudaSuccess)
      return CLIFFS_ERR_CUDA;
    // the scenarios' status words carry ST_STALL from the blocks that gave up
    for (cliffs_ctx* c : b->ctx)
      if (cudaMemsetAsync(c->status, 0, sizeof(unsigned), b->stream) != cudaSuccess) return CLIFFS_ERR_CUDA;
    if (cudaStreamSynchronize(b->stream) != cudaSuccess) return CLIFFS_ERR_CUDA;
  }
  return flags[1] ? CLIFFS_ERR_TIMEOUT : CLIFFS_OK;
}

int cliffs_batch_autotune(cliffs_batch* b, int32_t probe_steps, double* ms_per_step) {
  if (!b || probe_steps < 1) return CLIFFS_ERR_ARG;
  // snapshot of every context's state and max-wave fields
  std::vector<float*> saved;
  auto cleanup = [&]() {
    for (float* p : saved) cudaFree(p);
  };
  auto copy_state = [&](bool save) -> int {
    size_t k = 0;
    for (cliffs_ctx* c : b->ctx) {
      const size_t cells = (size_t)c->pitch * c->ny;
      float* fields[5] = {c->srf[c->cur], c->xu[c->cur], c->yv[c->cur], c->hmax, c->velmax};
      for (float* f : fields) {
        if (save) {
          float* p = nullptr;
          if (dalloc(&p, cells)) return CLIFFS_ERR_NOMEM;
          saved.push_back(p);
        }
        float* dst = save ? saved[k] : f;
        const float* src = save ? f : saved[k];
        if (cudaMemcpyAsync(dst, src, cells * sizeof(float), cudaMemcpyDeviceToDevice, b->stream) != cudaSuccess)
          return CLIFFS_ERR_CUDA;
        ++k;
      }
    }
    return cudaStreamSynchronize(b->stream) == cudaSuccess ? CLIFFS_OK : CLIFFS_ERR_CUDA;
  };
  struct Rise {  // a rising source's progress and the max-wave bookkeeping
    double el, w;
    bool on, pending, fresh;
  };
  std::vector<Rise> rise;
  for (cliffs_ctx* c : b->ctx) rise.push_back(Rise{c->rise_el, c->rise_w, c->rise_on, c->max_pending, c->max_fresh});
  auto restore_rise = [&]() {
    for (size_t k = 0; k < b->ctx.size(); ++k) {
      b->ctx[k]->rise_el = rise[k].el;
      b->ctx[k]->rise_w = rise[k].w;
      b->ctx[k]->rise_on = rise[k].on;
      b->ctx[k]->max_pending = rise[k].pending;
      b->ctx[k]->max_fresh = rise[k].fresh;
    }
  };
  int r = copy_state(true);
  if (r) {
    cleanup();
    return r;
  }
  // candidates: the schedule (persistent with 1..max resident blocks per SM,
  // graphs of 8 or 32 steps) and the tile shape (rows per x entry, 16-row
  // groups per y entry)
  std::vector<cliffs_batch_plan> cand;
  for (int k = 1; k <= b->max_ctas; ++k)
    for (int sh : {1, 2}) cand.push_back(cliffs_batch_plan{CLIFFS_BATCH_PERSISTENT, k, 32, sh, sh});
  for (int g : {8, 32})
    for (int sx : {1, 2, 4})
      for (int sy : {1, 2, 4}) cand.push_back(cliffs_batch_plan{CLIFFS_BATCH_GRAPH, 1, g, sx, sy});
  const cliffs_batch_plan keep = b->plan;
  cliffs_batch_plan best = keep;
  double best_ms = 1e300;
  const int64_t launches0 = b->launches;
  int64_t probed = 0;  // steps the probes ran
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (cudaEventCreate(&e0) || cudaEventCreate(&e1)) r = CLIFFS_ERR_CUDA;
  for (const cliffs_batch_plan& p : cand) {
    if (r) break;
    r = cliffs_batch_set_plan(b, &p);
    // a graph plan is timed on replays of its graph: the warm-up builds and
    // replays it once, the timed steps are whole graphs
    const bool graph = p.mode == CLIFFS_BATCH_GRAPH;
    const int warm = graph ? p.graph_steps : 1;
    const int steps = graph ? (std::max(probe_steps, p.graph_steps) + p.graph_steps - 1) / p.graph_steps * p.graph_steps
                            : probe_steps;
    if (!r) r = cliffs_batch_step(b, warm);
    if (!r && cudaEventRecord(e0, b->stream) != cudaSuccess) r = CLIFFS_ERR_CUDA;
    if (!r) r = cliffs_batch_step(b, steps);
    if (!r && cudaEventRecord(e1, b->stream) != cudaSuccess) r = CLIFFS_ERR_CUDA;
    float ms = 0;
    if (!r && (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess))
      r = CLIFFS_ERR_CUDA;
    if (!r && ms / steps < best_ms) {
      best_ms = ms / steps;
      best = p;
    }
    probed += warm + steps;
    if (!r) r = copy_state(false);
    restore_rise();
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  // the probes advanced the contexts' sweep counters; the restored state is
  // the one before the probes
  for (cliffs_ctx* c : b->ctx) c->sweeps -= (unsigned)(2 * probed);
  b->launches = launches0;
  cleanup();
  const int rp = cliffs_batch_set_plan(b, r ? &keep : &best);
  if (!r) r = rp;
  if (!r && ms_per_step) *ms_per_step = best_ms;
  return r;
}
