// mlp.cu -- the surrogate network of include/cliffs_surrogate.h.
//
// A ReLU multilayer perceptron, trained and evaluated on the GPU:
//   forward   H_{l+1} = relu(H_l W_l^T + b_l), out = H_d W_d^T + b_d
//   loss      mean over batch and outputs of (out - t)^2
//   backward  dW_l = dY_l^T H_l, db_l = sum_b dY_l, dH_l = dY_l W_l
//   update    Adam (FP32 master weights and moments), BF16 copies refreshed
// Every matrix product is gemm_tn below: C = A B^T with both operands in BF16
// and their reduction dimension contiguous, on the tensor cores through
// mma.sync m16n8k16 with FP32 accumulation; the epilogue adds the bias,
// applies the ReLU and writes the activations in the two layouts the backward
// pass reads (row-major for dH = dY W, transposed for dW = dY^T H).  Sizes are
// small (a few hundred to a few thousand rows); one 64x64 tile per block of
// four warps, K in steps of 32 through shared memory.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <random>
#include <vector>

#include "../../include/cliffs_gpu.h"
#include "../../include/cliffs_surrogate.h"
#include "decoder.cuh"

namespace cliffs_nn {

using bf16 = __nv_bfloat16;
constexpr int BM = 64, BN = 64, BK = 32, PAD = 8;

inline int pad16(int n) { return (n + 15) & ~15; }

struct Epi {
  const float* bias;  // [N] or null
  int relu;
  float* f32;         // [M][ldf] or null
  int ldf;
  bf16* b16;          // [M][ldb] or null
  int ldb;
  bf16* b16t;         // [N][ldt] (transposed) or null
  int ldt;
};

__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// C[M,N] = A[M,K] B[N,K]^T.  A and B are BF16 with K contiguous (leading
// dimensions lda, ldb, multiples of 8, 16-byte aligned rows); K is a multiple
// of 16 and both operands hold zeros in [K, round_up(K, 32)) or that range is
// past the end of the tile load (guarded).  M and N are arbitrary; M tiles
// run along grid x.  The products too small for gemm_tc (the first layer's
// 9 inputs, its weight gradient's 9 columns, batches under 128 rows) run
// here on mma.sync.
__global__ void __launch_bounds__(128) gemm_tn(int M, int N, int K, const bf16* __restrict__ A, int lda,
                                               const bf16* __restrict__ B, int ldb, Epi e) {
  __shared__ __align__(16) bf16 sA[BM][BK + PAD];
  __shared__ __align__(16) bf16 sB[BN][BK + PAD];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;
  const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
  const int g = lane >> 2, t = lane & 3;
  float acc[2][4][4];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int q = 0; q < 4; ++q) acc[i][j][q] = 0.f;
  const int ke = K;
  for (int k0 = 0; k0 < ke; k0 += BK) {
    // 64 rows x 32 columns per operand: 256 chunks of 8 elements (16 B)
    for (int c = tid; c < 256; c += 128) {
      const int r = c >> 2, col = (c & 3) * 8;
      const int gk = k0 + col;
      uint4 va = make_uint4(0, 0, 0, 0), vb = make_uint4(0, 0, 0, 0);
      if (m0 + r < M && gk < ke) va = *reinterpret_cast<const uint4*>(A + (size_t)(m0 + r) * lda + gk);
      if (n0 + r < N && gk < ke) vb = *reinterpret_cast<const uint4*>(B + (size_t)(n0 + r) * ldb + gk);
      *reinterpret_cast<uint4*>(&sA[r][col]) = va;
      *reinterpret_cast<uint4*>(&sB[r][col]) = vb;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < BK; kk += 16) {
      uint32_t af[2][4], bf[4][2];
#pragma unroll
      for (int i = 0; i < 2; ++i) {
        const int r = wm + i * 16;
        af[i][0] = *reinterpret_cast<const uint32_t*>(&sA[r + g][kk + 2 * t]);
        af[i][1] = *reinterpret_cast<const uint32_t*>(&sA[r + g + 8][kk + 2 * t]);
        af[i][2] = *reinterpret_cast<const uint32_t*>(&sA[r + g][kk + 2 * t + 8]);
        af[i][3] = *reinterpret_cast<const uint32_t*>(&sA[r + g + 8][kk + 2 * t + 8]);
      }
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int c = wn + j * 8;
        bf[j][0] = *reinterpret_cast<const uint32_t*>(&sB[c + g][kk + 2 * t]);
        bf[j][1] = *reinterpret_cast<const uint32_t*>(&sB[c + g][kk + 2 * t + 8]);
      }
#pragma unroll
      for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) mma_bf16(acc[i][j], af[i], bf[j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int row = m0 + wm + i * 16 + g + 8 * (q >> 1);
        const int col = n0 + wn + j * 8 + 2 * t + (q & 1);
        if (row >= M || col >= N) continue;
        float v = acc[i][j][q];
        if (e.bias) v += e.bias[col];
        if (e.relu) v = fmaxf(v, 0.f);
        if (e.f32) e.f32[(size_t)row * e.ldf + col] = v;
        const bf16 h = __float2bfloat16(v);
        if (e.b16) e.b16[(size_t)row * e.ldb + col] = h;
        if (e.b16t) e.b16t[(size_t)col * e.ldt + row] = h;
      }
}

}  // namespace cliffs_nn

#include "umma.cuh"

namespace cliffs_nn {

// Rows idx[r] (or r) of a row-major FP32 matrix into BF16 rows of length ld
// (columns past `cols` zero) and, when dst_t is set, the transpose [ld][ldt].
__global__ void k_pack(int rows, int cols, const float* __restrict__ src, const int* __restrict__ idx, bf16* dst,
                       int ld, bf16* dst_t, int ldt) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x, r = blockIdx.y;
  if (c >= ld || r >= rows) return;
  const int sr = idx ? idx[r] : r;
  const float v = c < cols ? src[(size_t)sr * cols + c] : 0.f;
  const bf16 h = __float2bfloat16(v);
  dst[(size_t)r * ld + c] = h;
  if (dst_t) dst_t[(size_t)c * ldt + r] = h;
}

__global__ void k_gather(int rows, int cols, const float* __restrict__ src, const int* __restrict__ idx, float* dst) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x, r = blockIdx.y;
  if (c >= cols || r >= rows) return;
  dst[(size_t)r * cols + c] = src[(size_t)(idx ? idx[r] : r) * cols + c];
}

// dY = scale (y - t) and per-block sums of (y - t)^2, in a fixed order.
__global__ void __launch_bounds__(256) k_mse(int n, const float* __restrict__ y, const float* __restrict__ tg,
                                             float* dy, float scale, float* part) {
  __shared__ float s[256];
  float acc = 0.f;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const float d = y[k] - tg[k];
    dy[k] = scale * d;
    acc += d * d;
  }
  s[threadIdx.x] = acc;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) s[threadIdx.x] += s[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = s[0];
}

// An FP32 gradient [B][N] into BF16 rows [B][ldb] (zero past N) and the
// transpose [N][ldt]; with H set, the ReLU derivative (H > 0) is applied and
// the FP32 gradient is overwritten with the masked one.
__global__ void k_grad_pack(int B, int N, float* dyf, const bf16* __restrict__ H, int ldH, bf16* dyb, int ldb,
                            bf16* dyt, int ldt) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x, r = blockIdx.y;
  if (c >= ldb || r >= B) return;
  float v = 0.f;
  if (c < N) {
    v = dyf[(size_t)r * N + c];
    if (H && !(__bfloat162float(H[(size_t)r * ldH + c]) > 0.f)) v = 0.f;
    dyf[(size_t)r * N + c] = v;
  }
  const bf16 h = __float2bfloat16(v);
  dyb[(size_t)r * ldb + c] = h;
  if (c < N) dyt[(size_t)c * ldt + r] = h;
}

// Adam with decoupled weight decay wd on an FP32 [rows][cols] parameter; W
// (BF16 [rows][ldW]) and Wt (BF16 [cols..][ldWt], transposed) are refreshed
// when given.
__global__ void k_adam(int rows, int cols, float* w, const float* __restrict__ gr, float* m, float* v, float lr,
                       float wd, float b1, float b2, float eps, float c1, float c2, bf16* W, int ldW, bf16* Wt,
                       int ldWt) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= rows * cols) return;
  const float gk = gr[k];
  const float mk = b1 * m[k] + (1.f - b1) * gk;
  const float vk = b2 * v[k] + (1.f - b2) * gk * gk;
  m[k] = mk;
  v[k] = vk;
  const float wk = w[k] * (1.f - lr * wd) - lr * (mk * c1) / (sqrtf(vk * c2) + eps);
  w[k] = wk;
  const int r = k / cols, c = k % cols;
  const bf16 h = __float2bfloat16(wk);
  if (W) W[(size_t)r * ldW + c] = h;
  if (Wt) Wt[(size_t)c * ldWt + r] = h;
}

}  // namespace cliffs_nn

using namespace cliffs_nn;

namespace {

template <typename T>
int dalloc(T** p, size_t n) {
  if (cudaMalloc((void**)p, std::max<size_t>(n, 1) * sizeof(T)) != cudaSuccess) {
    *p = nullptr;
    return 1;
  }
  return cudaMemset(*p, 0, std::max<size_t>(n, 1) * sizeof(T)) != cudaSuccess;
}

struct Layer {
  int rows = 0, cols = 0;  // W: rows x cols
  int kp = 0, rp = 0;      // cols and rows padded to 16
  float *w = nullptr, *b = nullptr, *gw = nullptr, *gb = nullptr;
  float *mw = nullptr, *vw = nullptr, *mb = nullptr, *vb = nullptr;
  bf16* W = nullptr;   // [rows][kp]
  bf16* Wt = nullptr;  // [kp][rp]
};

}  // namespace

struct cliffs_mlp {
  cliffs_mlp_desc d{};
  std::vector<Layer> L;
  cudaStream_t stream = nullptr;
  int cap = 0;                   // batch capacity of the activation buffers
  std::vector<bf16*> H, Ht;      // H[l]: input of layer l, [cap][kp_l]; Ht[l]: [kp_l][cap]
  float* out = nullptr;          // [cap][n_out]
  float* dyf = nullptr;          // [cap][maxN]
  float* dh = nullptr;           // [cap][maxN]
  bf16* dyb = nullptr;           // [cap][maxNp]
  bf16* dyt = nullptr;           // [maxNp][cap]
  float* part = nullptr;         // loss partial sums
  float* xs = nullptr;           // staged inputs / targets
  float* ts = nullptr;
  int staged = 0;
  int* idx = nullptr;
  int adam_t = 0;
  int64_t launches = 0;
  // dense layers, and the map decoder (d.map_side > 0): latent cells, latent
  // side, outputs of the last dense layer (n_out + latent), values per
  // sample of y and of the targets (n_out + map cells), channels per level
  int nd = 0;
  int lat = 0, s0 = 0, n_total = 0, n_y = 0, side2 = 0;
  int dc[4] = {0, 0, 0, 1};
  bf16* X[3] = {nullptr, nullptr, nullptr};  // decoder level inputs, NHWC
  float* map = nullptr;                      // [cap][side2]
  bf16* col = nullptr;                       // im2col [P][kp]
  float* dzf = nullptr;  // a level's output gradient, FP32 [P][Cout]
  bf16* dzb = nullptr;   // ... in BF16 [P][pad16(Cout)]
  float* dxf = nullptr;  // a level's input gradient (levels 1, 2)
  float* wpart = nullptr;  // partials of a weight gradient over chunks of pixels
  float* cpart = nullptr;  // partials of a bias gradient over chunks of pixels
  float* part2 = nullptr;  // map loss partial sums
  unsigned* err = nullptr;  // set by a tensor-core product whose wait ran out
  bool tc_failed = false;   // a tensor-core product could not be launched
};

namespace {

constexpr int kLossBlocks = 64;
constexpr int kMapLossBlocks = 1024;  // the map loss: B x side^2 values

void free_decoder(cliffs_mlp* m) {
  void* p[] = {m->X[0], m->X[1], m->X[2], m->map, m->col, m->dzf, m->dzb, m->dxf, m->wpart, m->cpart, m->part2};
  for (void* q : p)
    if (q) cudaFree(q);
  m->X[0] = m->X[1] = m->X[2] = nullptr;
  m->col = m->dzb = nullptr;
  m->map = m->dzf = m->dxf = m->wpart = m->cpart = m->part2 = nullptr;
}

void free_all(cliffs_mlp* m) {
  free_decoder(m);
  for (Layer& l : m->L) {
    void* p[] = {l.w, l.b, l.gw, l.gb, l.mw, l.vw, l.mb, l.vb, l.W, l.Wt};
    for (void* q : p)
      if (q) cudaFree(q);
  }
  for (bf16* p : m->H)
    if (p) cudaFree(p);
  for (bf16* p : m->Ht)
    if (p) cudaFree(p);
  void* p[] = {m->out, m->dyf, m->dh, m->dyb, m->dyt, m->part, m->xs, m->ts, m->idx, m->err};
  for (void* q : p)
    if (q) cudaFree(q);
  m->err = nullptr;
  m->H.clear();
  m->Ht.clear();
  m->out = m->dyf = m->dh = m->part = m->xs = m->ts = nullptr;
  m->dyb = m->dyt = nullptr;
  m->idx = nullptr;
}

int max_n(const cliffs_mlp* m) { return std::max(m->d.width, m->n_total); }

// Decoder level l (0..2): input side, input and output channels, im2col width.
struct Level {
  int lvl, S, cin, cout, K, kp;
};
Level level(const cliffs_mlp* m, int l) {
  Level v;
  v.lvl = l;
  v.S = m->s0 << l;
  v.cin = m->dc[l];
  v.cout = m->dc[l + 1];
  v.K = 9 * v.cin;
  v.kp = pad16(v.K);
  return v;
}
constexpr int kDwChunk = 512;  // least output pixels per partial of a decoder weight gradient

// Output pixels per partial of a level's weight gradient (P pixels) (a multiple of
// kStage; at most ~2048 partials), and the number of partials.
int dw_chunk(long long P) {
  const long long c = std::max<long long>(kDwChunk, ((P + 2047) / 2048 + kStage - 1) / kStage * kStage);
  return (int)c;
}
int dw_blocks(long long P) { return (int)((P + dw_chunk(P) - 1) / dw_chunk(P)); }

// The direct kernels' output-channel class: CO >= cout of 1, 8, 16, 32, 64.
int co_class(int cout) { return cout <= 1 ? 1 : cout <= 8 ? 8 : cout <= 16 ? 16 : cout <= 32 ? 32 : 64; }

// Activation buffers for batches up to cap.
int ensure_cap(cliffs_mlp* m, int cap) {
  if (cap <= m->cap) return CLIFFS_OK;
  // the decoder kernels index pixels and values in 32 bits: at most 64
  // channels at a quarter of the map's cells, 16 values per map cell
  if (m->d.map_side > 0 && (long long)cap * m->side2 * 16 >= (1ll << 31)) return CLIFFS_ERR_ARG;
  for (bf16* p : m->H)
    if (p) cudaFree(p);
  for (bf16* p : m->Ht)
    if (p) cudaFree(p);
  void* p[] = {m->out, m->dyf, m->dh, m->dyb, m->dyt, m->part};
  for (void* q : p)
    if (q) cudaFree(q);
  m->H.assign(m->nd, nullptr);  // inputs of the dense layers
  m->Ht.assign(m->nd, nullptr);
  const int mn = max_n(m), mnp = pad16(mn);
  for (int l = 0; l < m->nd; ++l) {
    if (dalloc(&m->H[l], (size_t)cap * m->L[l].kp) || dalloc(&m->Ht[l], (size_t)m->L[l].kp * cap))
      return CLIFFS_ERR_NOMEM;
  }
  if (dalloc(&m->out, (size_t)cap * m->n_total) || dalloc(&m->dyf, (size_t)cap * mn) ||
      dalloc(&m->dh, (size_t)cap * mn) || dalloc(&m->dyb, (size_t)cap * mnp) || dalloc(&m->dyt, (size_t)mnp * cap) ||
      dalloc(&m->part, kLossBlocks))
    return CLIFFS_ERR_NOMEM;
  if (m->d.map_side > 0) {
    free_decoder(m);
    size_t col = 0, dz = 0, dzp = 0, dx = 0, wp = 0, bp = 0;
    for (int l = 0; l < 3; ++l) {
      const Level v = level(m, l);
      const size_t P = (size_t)cap * 4 * v.S * v.S;
      if (v.cout >= 16) col = std::max(col, P * v.kp);  // im2col of the tensor-core levels
      dz = std::max(dz, P * v.cout);
      dzp = std::max(dzp, P * v.cout);
      if (l > 0) dx = std::max(dx, (size_t)cap * v.S * v.S * v.cin);
      wp = std::max(wp, (size_t)dw_blocks((long long)P) * v.cout * v.K);
      bp = std::max(bp, (size_t)dw_blocks((long long)P) * v.cout);
      if (dalloc(&m->X[l], (size_t)cap * v.S * v.S * v.cin)) return CLIFFS_ERR_NOMEM;
    }
    if (dalloc(&m->map, (size_t)cap * m->side2) || dalloc(&m->col, col) ||
        dalloc(&m->dzf, std::max(dz, dx)) || dalloc(&m->dzb, dzp) ||
        dalloc(&m->dxf, std::max(dz, dx)) || dalloc(&m->wpart, wp) || dalloc(&m->cpart, bp) ||
        dalloc(&m->part2, kMapLossBlocks))
      return CLIFFS_ERR_NOMEM;
  }
  m->cap = cap;
  return CLIFFS_OK;
}

PFN_cuTensorMapEncodeTiled_v12000 g_encode_bf16 = nullptr;

// A 2-D BF16 tensor map over rows x k (k contiguous, rows ld elements apart)
// with a box of 64 x box_rows in the 128-byte swizzled layout; elements
// outside read 0.
bool bf16_map(CUtensorMap* map, const bf16* base, int rows, int k, int ld, int box_rows) {
  if (!g_encode_bf16) {
    cudaDriverEntryPointQueryResult q;
    void* fn = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !fn)
      return false;
    g_encode_bf16 = (PFN_cuTensorMapEncodeTiled_v12000)fn;
  }
  cuuint64_t dims[2] = {(cuuint64_t)k, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)ld * sizeof(bf16)};
  cuuint32_t box[2] = {(cuuint32_t)umma::BK, (cuuint32_t)box_rows};
  cuuint32_t es[2] = {1, 1};
  return g_encode_bf16(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<bf16*>(base), dims, strides, box, es,
                       CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                       CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int BN>
bool gemm_tc_launch(cliffs_mlp* m, int M, int N, int K, const bf16* A, int lda, const bf16* B, int ldb,
                    const Epi& e) {
  static bool attr = false;
  if (!attr) {
    if (cudaFuncSetAttribute(gemm_tc<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)gemm_tc_smem<BN>()) !=
        cudaSuccess)
      return false;
    attr = true;
  }
  CUtensorMap ta, tb;
  if (!bf16_map(&ta, A, M, K, lda, umma::BM) || !bf16_map(&tb, B, N, K, ldb, BN)) return false;
  const dim3 grid((M + umma::BM - 1) / umma::BM, (N + BN - 1) / BN);
  gemm_tc<BN><<<grid, umma::THREADS, gemm_tc_smem<BN>(), m->stream>>>(ta, tb, M, N, K, e, m->err);
  ++m->launches;
  return cudaGetLastError() == cudaSuccess;
}

// C = A B^T.  Products of at least 128 rows, 16 columns and a reduction of
// 64 whose operands suit the tensor-memory path (16-byte aligned rows,
// 128-byte aligned bases) run as gemm_tc, with the widest tile of 16, 64 or
// 128 columns that N fills; the others (small batches, the first layer's 9
// inputs) run as gemm_tn.
void gemm(cliffs_mlp* m, int M, int N, int K, const bf16* A, int lda, const bf16* B, int ldb, const Epi& e) {
  // every tensor-map box lies within its operand's extent: M >= 128 rows,
  // K >= 64, and a tile width of at most N (16, 64 or 128)
  const bool tc_ok = M >= umma::BM && N >= 16 && K >= umma::BK && lda % 8 == 0 && ldb % 8 == 0 &&
                     ((uintptr_t)A % 128) == 0 && ((uintptr_t)B % 128) == 0;
  if (tc_ok) {
    const bool launched = N >= 128  ? gemm_tc_launch<128>(m, M, N, K, A, lda, B, ldb, e)
                          : N >= 64 ? gemm_tc_launch<64>(m, M, N, K, A, lda, B, ldb, e)
                                    : gemm_tc_launch<16>(m, M, N, K, A, lda, B, ldb, e);
    if (!launched) m->tc_failed = true;  // reported by the call (CLIFFS_ERR_CUDA)
    return;
  }
  const dim3 grid((M + BM - 1) / BM, (N + BN - 1) / BN);
  gemm_tn<<<grid, 128, 0, m->stream>>>(M, N, K, A, lda, B, ldb, e);
  ++m->launches;
}

// Blocks of 256 threads covering n elements.
inline unsigned blocks256(long long n) { return (unsigned)((n + 255) / 256); }

// Shared memory above the default 48 KB for a kernel (once per kernel).
template <typename Kernel>
void smem_limit(Kernel* k, size_t bytes) {
  if (bytes > 48 * 1024) cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

template <int CO>
void dec_conv_launch(cliffs_mlp* m, int B, const Level& v, const Layer& y, bf16* out16, float* out32) {
  const long long P = (long long)B * 4 * v.S * v.S;
  const size_t sh = (size_t)9 * v.cin * CO * 4;
  smem_limit(k_dec_conv<CO>, sh);
  k_dec_conv<CO><<<blocks256(P), 256, sh, m->stream>>>(B, v.S, v.cin, v.cout, m->X[v.lvl], y.W, y.kp, y.b, out16,
                                                       out32);
}

template <int CO>
void dec_dw_launch(cliffs_mlp* m, int B, const Level& v) {
  constexpr int G = dec_group<CO>();
  const long long P = (long long)B * 4 * v.S * v.S;
  const int KG = v.K / G, KGb = std::min(KG, 256), threads = KGb * std::max(1, 256 / KGb);
  const size_t sh = dec_dw_smem<CO>(v.cin);
  smem_limit(k_dec_dw<CO>, sh);
  const dim3 grid(dw_blocks(P), (KG + KGb - 1) / KGb);
  k_dec_dw<CO><<<grid, threads, sh, m->stream>>>(B, v.S, v.cin, v.cout, m->dzb, v.cout, m->X[v.lvl],
                                                 dw_chunk(P), m->wpart, m->cpart);
}

template <int CO>
void dec_dx_launch(cliffs_mlp* m, int B, const Level& v, const Layer& y, float* dx, int ld, int col0) {
  constexpr int G = dec_group<CO>();
  const long long n = (long long)B * v.S * v.S * (v.cin / G);
  const size_t sh = (size_t)9 * v.cin * CO * 4;
  smem_limit(k_dec_dx<CO>, sh);
  k_dec_dx<CO><<<blocks256(n), 256, sh, m->stream>>>(B, v.S, v.cin, v.cout, m->dzb, v.cout, y.W, y.kp,
                                                     m->X[v.lvl], dx, ld, col0);
}

// The map decoder's forward pass for rows [0, B): latent columns of out -> map.
void decoder_forward(cliffs_mlp* m, int B) {
  k_dec_input<<<blocks256((long long)B * m->lat), 256, 0, m->stream>>>(B, m->lat, m->out, m->n_total, m->d.n_out,
                                                                       m->X[0]);
  ++m->launches;
  for (int l = 0; l < 3; ++l) {
    const Level v = level(m, l);
    const Layer& y = m->L[m->nd + l];
    bf16* out16 = l < 2 ? m->X[l + 1] : nullptr;  // ReLU and BF16 NHWC, or the FP32 map
    float* out32 = l < 2 ? nullptr : m->map;
    if (v.cout < 16) {  // below the tensor cores' narrowest tile: direct
      if (v.cout == 1)
        dec_conv_launch<1>(m, B, v, y, out16, out32);
      else
        dec_conv_launch<8>(m, B, v, y, out16, out32);
      ++m->launches;
      continue;
    }
    const int P = B * 4 * v.S * v.S;
    k_im2col_up<<<(P + 7) / 8, dim3(32, 8), 0, m->stream>>>(B, v.S, v.cin, m->X[l], v.kp, m->col);
    ++m->launches;
    Epi e{};
    e.bias = y.b;
    if (l < 2) {
      e.relu = 1;
      e.b16 = out16;
      e.ldb = v.cout;
    } else {
      e.f32 = out32;
      e.ldf = 1;
    }
    gemm(m, P, v.cout, v.kp, m->col, v.kp, y.W, y.kp, e);
  }
}

// The map decoder's backward pass: the map gradient is in dzf ([B][side2]);
// the gradients of the decoder's weights and biases, and the latent's into
// dyf columns [n_out, n_total).
void decoder_backward(cliffs_mlp* m, int B) {
  for (int l = 2; l >= 0; --l) {
    const Level v = level(m, l);
    Layer& y = m->L[m->nd + l];
    const int P = B * 4 * v.S * v.S;
    // the output gradient in BF16 rows of cout values (ReLU masks applied by
    // the level above's input gradient)
    k_to_bf16<<<blocks256((long long)P * v.cout), 256, 0, m->stream>>>(P * v.cout, m->dzf, m->dzb);
    // weight and bias gradients: partial sums over chunks of pixels, then
    // over the chunks in order
    switch (co_class(v.cout)) {
      case 1: dec_dw_launch<1>(m, B, v); break;
      case 8: dec_dw_launch<8>(m, B, v); break;
      case 16: dec_dw_launch<16>(m, B, v); break;
      case 32: dec_dw_launch<32>(m, B, v); break;
      default: dec_dw_launch<64>(m, B, v); break;
    }
    const int nb = dw_blocks(P);
    k_reduce_wgrad<<<(v.cout * v.K + 31) / 32, 32 * kStrands, 0, m->stream>>>(v.cout, v.K, v.K, nb, m->wpart, y.gw);
    k_reduce_wgrad<<<(v.cout + 31) / 32, 32 * kStrands, 0, m->stream>>>(1, v.cout, v.cout, nb, m->cpart, y.gb);
    // input gradient, masked by the level input's ReLU; level 0's goes to
    // the latent columns of the dense output gradient
    float* dx = l > 0 ? m->dxf : m->dyf;
    const int ld = l > 0 ? v.S * v.S * v.cin : m->n_total, col0 = l > 0 ? 0 : m->d.n_out;
    switch (co_class(v.cout)) {
      case 1: dec_dx_launch<1>(m, B, v, y, dx, ld, col0); break;
      case 8: dec_dx_launch<8>(m, B, v, y, dx, ld, col0); break;
      case 16: dec_dx_launch<16>(m, B, v, y, dx, ld, col0); break;
      case 32: dec_dx_launch<32>(m, B, v, y, dx, ld, col0); break;
      default: dec_dx_launch<64>(m, B, v, y, dx, ld, col0); break;
    }
    m->launches += 5;
    if (l > 0) std::swap(m->dzf, m->dxf);  // the input gradient is the next level's output gradient
  }
}

// Forward pass of rows [0, B) staged in H[0] (and Ht[0]); out gets the result.
void forward(cliffs_mlp* m, int B) {
  const int nl = m->nd;
  for (int l = 0; l < nl; ++l) {
    const Layer& y = m->L[l];
    Epi e{};
    e.bias = y.b;
    if (l < nl - 1) {
      e.relu = 1;
      e.b16 = m->H[l + 1];
      e.ldb = m->L[l + 1].kp;
      e.b16t = m->Ht[l + 1];
      e.ldt = m->cap;
    } else {
      e.f32 = m->out;
      e.ldf = m->n_total;
    }
    gemm(m, B, y.rows, y.kp, m->H[l], y.kp, y.W, y.kp, e);
  }
  if (m->d.map_side > 0) decoder_forward(m, B);
}

void stage_inputs(cliffs_mlp* m, int B, const float* x_dev, const int* idx) {
  const int kp0 = m->L[0].kp;
  k_pack<<<dim3((kp0 + 127) / 128, B), 128, 0, m->stream>>>(B, m->d.n_in, x_dev, idx, m->H[0], kp0, m->Ht[0], m->cap);
  ++m->launches;
}

// Loss and gradients of the batch staged by stage_inputs with targets t_dev
// (rows idx); returns the sum of squared errors through *part on the device.
void backward(cliffs_mlp* m, int B, const float* t_dev, const int* idx) {
  const int nl = m->nd;
  const int no = m->d.n_out;
  if (m->d.map_side > 0) {
    // dense outputs: dY of their columns; the map: its gradient, then the
    // decoder's backward pass fills the latent columns of dY
    k_mse_block<<<kLossBlocks, 256, 0, m->stream>>>(B, no, m->out, m->n_total, 0, t_dev, m->n_y, 0, idx, m->dyf,
                                                    m->n_total, 0, 2.f / ((float)B * no), m->part);
    k_mse_block<<<kMapLossBlocks, 256, 0, m->stream>>>(B, m->side2, m->map, m->side2, 0, t_dev, m->n_y, no, idx,
                                                    m->dzf, m->side2, 0, 2.f / ((float)B * m->side2), m->part2);
    m->launches += 2;
    decoder_backward(m, B);
  } else {
    // targets of the batch into dh (scratch), then dY of the output layer
    k_gather<<<dim3((no + 127) / 128, B), 128, 0, m->stream>>>(B, no, t_dev, idx, m->dh);
    k_mse<<<kLossBlocks, 256, 0, m->stream>>>(B * no, m->out, m->dh, m->dyf, 2.f / ((float)B * no), m->part);
    m->launches += 2;
  }
  for (int l = nl - 1; l >= 0; --l) {
    const Layer& y = m->L[l];
    const int N = y.rows, Np = y.rp;
    // dY of this layer: BF16 rows and transpose; ReLU derivative for hidden layers
    const bf16* Hmask = l < nl - 1 ? m->H[l + 1] : nullptr;
    const int ldH = l < nl - 1 ? m->L[l + 1].kp : 0;
    k_grad_pack<<<dim3((Np + 127) / 128, B), 128, 0, m->stream>>>(B, N, m->dyf, Hmask, ldH, m->dyb, Np, m->dyt,
                                                                  m->cap);
    k_reduce_wgrad<<<(N + 31) / 32, 32 * kStrands, 0, m->stream>>>(1, N, N, B, m->dyf, y.gb);  // column sums
    m->launches += 2;
    // dW = dY^T H_l: (N x B) (B x cols), reduction over the batch
    Epi ew{};
    ew.f32 = y.gw;
    ew.ldf = y.cols;
    gemm(m, N, y.cols, B, m->dyt, m->cap, m->Ht[l], m->cap, ew);
    // dH_l = dY W: (B x Np) (Np x kp), the input gradient of the layer below
    if (l > 0) {
      Epi eh{};
      eh.f32 = m->dyf;  // read above; the next layer's dY is built in place
      eh.ldf = y.cols;
      gemm(m, B, y.cols, Np, m->dyb, Np, y.Wt, Np, eh);
    }
  }
}

void adam(cliffs_mlp* m, float lr, float wd) {
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  ++m->adam_t;
  const float c1 = 1.f / (1.f - std::pow(b1, (float)m->adam_t));
  const float c2 = 1.f / (1.f - std::pow(b2, (float)m->adam_t));
  for (Layer& y : m->L) {
    const int nw = y.rows * y.cols;
    k_adam<<<(nw + 255) / 256, 256, 0, m->stream>>>(y.rows, y.cols, y.w, y.gw, y.mw, y.vw, lr, wd, b1, b2, eps, c1,
                                                    c2, y.W, y.kp, y.Wt, y.rp);
    k_adam<<<(y.rows + 255) / 256, 256, 0, m->stream>>>(y.rows, 1, y.b, y.gb, y.mb, y.vb, lr, 0.f, b1, b2, eps, c1,
                                                        c2, nullptr, 0, nullptr, 0);
    m->launches += 2;
  }
}

// The BF16 copies of layer weights from the FP32 master.
int refresh_bf16(cliffs_mlp* m, Layer& y) {
  std::vector<float> w((size_t)y.rows * y.cols);
  if (cudaMemcpy(w.data(), y.w, w.size() * 4, cudaMemcpyDeviceToHost) != cudaSuccess) return CLIFFS_ERR_CUDA;
  std::vector<bf16> W((size_t)y.rows * y.kp, __float2bfloat16(0.f)), Wt((size_t)y.kp * y.rp, __float2bfloat16(0.f));
  for (int r = 0; r < y.rows; ++r)
    for (int c = 0; c < y.cols; ++c) {
      const bf16 h = __float2bfloat16(w[(size_t)r * y.cols + c]);
      W[(size_t)r * y.kp + c] = h;
      Wt[(size_t)c * y.rp + r] = h;
    }
  if (cudaMemcpy(y.W, W.data(), W.size() * sizeof(bf16), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(y.Wt, Wt.data(), Wt.size() * sizeof(bf16), cudaMemcpyHostToDevice) != cudaSuccess)
    return CLIFFS_ERR_CUDA;
  (void)m;
  return CLIFFS_OK;
}

int stage_data(cliffs_mlp* m, int n, const float* x, const float* t) {
  if (n > m->staged) {
    if (m->xs) cudaFree(m->xs);
    if (m->ts) cudaFree(m->ts);
    if (m->idx) cudaFree(m->idx);
    m->xs = m->ts = nullptr;
    m->idx = nullptr;
    m->staged = 0;
    if (dalloc(&m->xs, (size_t)n * m->d.n_in) || dalloc(&m->ts, (size_t)n * m->n_y) || dalloc(&m->idx, n))
      return CLIFFS_ERR_NOMEM;
    m->staged = n;
  }
  if (cudaMemcpyAsync(m->xs, x, (size_t)n * m->d.n_in * 4, cudaMemcpyHostToDevice, m->stream) != cudaSuccess)
    return CLIFFS_ERR_CUDA;
  if (t && cudaMemcpyAsync(m->ts, t, (size_t)n * m->n_y * 4, cudaMemcpyHostToDevice, m->stream) != cudaSuccess)
    return CLIFFS_ERR_CUDA;
  return CLIFFS_OK;
}

// The products' status since the last call: CLIFFS_ERR_TIMEOUT when a
// tensor-core product's wait ran out (cleared), CLIFFS_ERR_CUDA when one could
// not be launched; synchronises.
int products_status(cliffs_mlp* m) {
  unsigned e = 0;
  if (cudaMemcpyAsync(&e, m->err, sizeof(e), cudaMemcpyDeviceToHost, m->stream) != cudaSuccess ||
      cudaStreamSynchronize(m->stream) != cudaSuccess)
    return CLIFFS_ERR_CUDA;
  if (e) {
    cudaMemsetAsync(m->err, 0, sizeof(unsigned), m->stream);
    return CLIFFS_ERR_TIMEOUT;
  }
  if (m->tc_failed) {
    m->tc_failed = false;
    return CLIFFS_ERR_CUDA;
  }
  return CLIFFS_OK;
}

float loss_of(cliffs_mlp* m, int B) {
  float part[kLossBlocks];
  std::vector<float> part2(kMapLossBlocks);
  cudaMemcpyAsync(part, m->part, sizeof(part), cudaMemcpyDeviceToHost, m->stream);
  if (m->d.map_side > 0)
    cudaMemcpyAsync(part2.data(), m->part2, part2.size() * sizeof(float), cudaMemcpyDeviceToHost, m->stream);
  cudaStreamSynchronize(m->stream);
  double s = 0, s2 = 0;
  for (float p : part) s += p;
  if (m->d.map_side > 0)
    for (float p : part2) s2 += p;
  double loss = s / ((double)B * m->d.n_out);
  if (m->d.map_side > 0) loss += s2 / ((double)B * m->side2);
  return (float)loss;
}

}  // namespace

int cliffs_mlp_create(const cliffs_mlp_desc* d, cliffs_mlp** out) {
  if (!d || !out || d->n_in < 1 || d->n_in > 16 || d->width < 16 || d->width % 16 || d->width > 4096 ||
      d->depth < 1 || d->depth > 16 || d->n_out < 1 || d->n_out > 16384)
    return CLIFFS_ERR_ARG;
  if (d->map_side < 0 || d->map_side % 8 || d->map_side > 512) return CLIFFS_ERR_ARG;
  if (d->map_side > 0)
    for (int c : d->map_ch)
      if (c < 8 || c % 8 || c > 64) return CLIFFS_ERR_ARG;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) return CLIFFS_ERR_DEVICE;
  auto* m = new cliffs_mlp;
  m->d = *d;
  m->nd = d->depth + 1;
  if (d->map_side > 0) {
    m->s0 = d->map_side / 8;
    m->lat = m->s0 * m->s0 * d->map_ch[0];
    m->side2 = d->map_side * d->map_side;
    for (int k = 0; k < 3; ++k) m->dc[k] = d->map_ch[k];
    m->dc[3] = 1;
  }
  m->n_total = d->n_out + m->lat;
  m->n_y = d->n_out + m->side2;
  auto fail = [&](int r) {
    free_all(m);
    if (m->stream) cudaStreamDestroy(m->stream);
    delete m;
    return r;
  };
  if (cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking) != cudaSuccess) return fail(CLIFFS_ERR_CUDA);
  if (dalloc(&m->err, 1)) return fail(CLIFFS_ERR_NOMEM);
  std::mt19937_64 rng(d->seed);
  const int nlayers = m->nd + (d->map_side > 0 ? 3 : 0);
  for (int l = 0; l < nlayers; ++l) {
    Layer y;
    const bool conv = l >= m->nd;
    if (conv) {  // decoder level l - nd: [Cout][9 Cin]
      y.cols = 9 * m->dc[l - m->nd];
      y.rows = m->dc[l - m->nd + 1];
    } else {
      y.cols = l == 0 ? d->n_in : d->width;
      y.rows = l == d->depth ? m->n_total : d->width;
    }
    y.kp = pad16(y.cols);
    y.rp = pad16(y.rows);
    const size_t nw = (size_t)y.rows * y.cols;
    if (dalloc(&y.w, nw) || dalloc(&y.b, y.rows) || dalloc(&y.gw, nw) || dalloc(&y.gb, y.rows) ||
        dalloc(&y.mw, nw) || dalloc(&y.vw, nw) || dalloc(&y.mb, y.rows) || dalloc(&y.vb, y.rows) ||
        dalloc(&y.W, (size_t)y.rows * y.kp) || dalloc(&y.Wt, (size_t)y.kp * y.rp)) {
      m->L.push_back(y);
      return fail(CLIFFS_ERR_NOMEM);
    }
    // He uniform for layers followed by a ReLU (the latent passes one),
    // Glorot-like for the linear outputs
    const bool relu_after = conv ? l < nlayers - 1 : (l < d->depth || d->map_side > 0);
    const double a = relu_after ? std::sqrt(6.0 / y.cols) : std::sqrt(3.0 / y.cols);
    std::uniform_real_distribution<double> U(-a, a);
    std::vector<float> w(nw);
    for (float& v : w) v = (float)U(rng);
    if (cudaMemcpy(y.w, w.data(), nw * 4, cudaMemcpyHostToDevice) != cudaSuccess) {
      m->L.push_back(y);
      return fail(CLIFFS_ERR_CUDA);
    }
    m->L.push_back(y);
    if (refresh_bf16(m, m->L.back())) return fail(CLIFFS_ERR_CUDA);
  }
  *out = m;
  return CLIFFS_OK;
}

void cliffs_mlp_destroy(cliffs_mlp* m) {
  if (!m) return;
  cudaStreamSynchronize(m->stream);
  free_all(m);
  cudaStreamDestroy(m->stream);
  delete m;
}

int cliffs_mlp_layers(const cliffs_mlp* m, int32_t* n) {
  if (!m || !n) return CLIFFS_ERR_ARG;
  *n = (int32_t)m->L.size();
  return CLIFFS_OK;
}

int cliffs_mlp_shape(const cliffs_mlp* m, int32_t l, int32_t* rows, int32_t* cols) {
  if (!m || l < 0 || l >= (int)m->L.size() || !rows || !cols) return CLIFFS_ERR_ARG;
  *rows = m->L[l].rows;
  *cols = m->L[l].cols;
  return CLIFFS_OK;
}

static float* param_ptr(const cliffs_mlp* m, int l, int which, int64_t* n) {
  const Layer& y = m->L[l];
  *n = which == 0 || which == 2 ? (int64_t)y.rows * y.cols : y.rows;
  switch (which) {
    case 0: return y.w;
    case 1: return y.b;
    case 2: return y.gw;
    case 3: return y.gb;
  }
  return nullptr;
}

int cliffs_mlp_get(const cliffs_mlp* m, int32_t l, int32_t which, float* host, int64_t n) {
  if (!m || l < 0 || l >= (int)m->L.size() || which < 0 || which > 3 || !host) return CLIFFS_ERR_ARG;
  int64_t cnt = 0;
  float* p = param_ptr(m, l, which, &cnt);
  if (n != cnt) return CLIFFS_ERR_ARG;
  if (cudaStreamSynchronize(m->stream) != cudaSuccess || cudaMemcpy(host, p, cnt * 4, cudaMemcpyDeviceToHost))
    return CLIFFS_ERR_CUDA;
  return CLIFFS_OK;
}

int cliffs_mlp_set(cliffs_mlp* m, int32_t l, int32_t which, const float* host, int64_t n) {
  if (!m || l < 0 || l >= (int)m->L.size() || which < 0 || which > 1 || !host) return CLIFFS_ERR_ARG;
  int64_t cnt = 0;
  float* p = param_ptr(m, l, which, &cnt);
  if (n != cnt) return CLIFFS_ERR_ARG;
  if (cudaStreamSynchronize(m->stream) != cudaSuccess || cudaMemcpy(p, host, cnt * 4, cudaMemcpyHostToDevice))
    return CLIFFS_ERR_CUDA;
  return which == 0 ? refresh_bf16(m, m->L[l]) : CLIFFS_OK;
}

int cliffs_mlp_predict(cliffs_mlp* m, int32_t batch, const float* x, float* y) {
  if (!m || batch < 1 || !x || !y) return CLIFFS_ERR_ARG;
  // the decoder's buffers grow with the batch: predict maps in chunks of 256
  const int chunk = m->d.map_side > 0 ? 256 : 4096;
  int r = ensure_cap(m, pad16(std::min<int>(batch, chunk)));
  if (!r) r = stage_data(m, batch, x, nullptr);
  for (int s = 0; !r && s < batch; s += chunk) {
    const int B = std::min(chunk, batch - s);
    stage_inputs(m, B, m->xs + (size_t)s * m->d.n_in, nullptr);
    forward(m, B);
    // rows of n_y: the dense outputs, then the map
    float* yr = y + (size_t)s * m->n_y;
    if (cudaMemcpy2DAsync(yr, (size_t)m->n_y * 4, m->out, (size_t)m->n_total * 4, (size_t)m->d.n_out * 4, B,
                          cudaMemcpyDeviceToHost, m->stream) != cudaSuccess)
      r = CLIFFS_ERR_CUDA;
    if (!r && m->d.map_side > 0 &&
        cudaMemcpy2DAsync(yr + m->d.n_out, (size_t)m->n_y * 4, m->map, (size_t)m->side2 * 4, (size_t)m->side2 * 4,
                          B, cudaMemcpyDeviceToHost, m->stream) != cudaSuccess)
      r = CLIFFS_ERR_CUDA;
  }
  if (cudaStreamSynchronize(m->stream) != cudaSuccess && !r) r = CLIFFS_ERR_CUDA;
  if (!r && cudaGetLastError() != cudaSuccess) r = CLIFFS_ERR_CUDA;
  if (!r) r = products_status(m);
  return r;
}

int cliffs_mlp_gradients(cliffs_mlp* m, int32_t batch, const float* x, const float* t, float* loss) {
  if (!m || batch < 16 || batch % 16 || !x || !t) return CLIFFS_ERR_ARG;
  int r = ensure_cap(m, batch);
  if (!r) r = stage_data(m, batch, x, t);
  if (r) return r;
  stage_inputs(m, batch, m->xs, nullptr);
  forward(m, batch);
  backward(m, batch, m->ts, nullptr);
  const float l = loss_of(m, batch);
  if (loss) *loss = l;
  if (cudaGetLastError() != cudaSuccess) return CLIFFS_ERR_CUDA;
  return products_status(m);
}

int cliffs_mlp_train(cliffs_mlp* m, int32_t n, const float* x, const float* t, int32_t epochs, int32_t batch,
                     float lr, float weight_decay, uint64_t seed, float* losses) {
  if (!m || n < batch || batch < 16 || batch % 16 || epochs < 1 || !x || !t || !(lr > 0) || !(weight_decay >= 0))
    return CLIFFS_ERR_ARG;
  int r = ensure_cap(m, batch);
  if (!r) r = stage_data(m, n, x, t);
  if (r) return r;
  std::mt19937_64 rng(seed);
  std::vector<int> perm(n);
  for (int k = 0; k < n; ++k) perm[k] = k;
  const int per_epoch = n / batch;
  const int total = per_epoch * epochs;
  int it = 0;
  for (int e = 0; e < epochs && !r; ++e) {
    std::shuffle(perm.begin(), perm.end(), rng);
    if (cudaMemcpyAsync(m->idx, perm.data(), (size_t)n * 4, cudaMemcpyHostToDevice, m->stream) != cudaSuccess) {
      r = CLIFFS_ERR_CUDA;
      break;
    }
    double sum = 0;
    for (int b = 0; b < per_epoch; ++b, ++it) {
      const int* idx = m->idx + (size_t)b * batch;
      stage_inputs(m, batch, m->xs, idx);
      forward(m, batch);
      backward(m, batch, m->ts, idx);
      const double frac = (double)it / std::max(1, total - 1);
      const float lr_it = (float)(lr * (0.05 + 0.95 * 0.5 * (1.0 + std::cos(M_PI * frac))));
      adam(m, lr_it, weight_decay);
      if (losses) sum += loss_of(m, batch);
    }
    if (losses) losses[e] = (float)(sum / per_epoch);
    // the permutation buffer is rewritten next epoch: the stream must be done with it
    if (cudaStreamSynchronize(m->stream) != cudaSuccess) r = CLIFFS_ERR_CUDA;
  }
  if (!r && cudaGetLastError() != cudaSuccess) r = CLIFFS_ERR_CUDA;
  if (!r) r = products_status(m);
  return r;
}

int cliffs_mlp_launch_count(const cliffs_mlp* m, int64_t* n) {
  if (!m || !n) return CLIFFS_ERR_ARG;
  *n = m->launches;
  return CLIFFS_OK;
}
