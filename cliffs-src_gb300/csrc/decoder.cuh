// decoder.cuh -- the map decoder of the surrogate network (mlp.cu).
//
// The network's last dense layer emits, besides its dense outputs, a latent
// grid of S0 x S0 cells with C0 channels (row-major, channels fastest: NHWC).
// The decoder takes it through a ReLU and then through levels that each
// upsample by 2 (nearest neighbour) and apply a 3x3 convolution with zero
// padding and a bias; every level but the last applies a ReLU, the last has
// one output channel: the map.  Activations are BF16 in NHWC, weights BF16 as
// [Cout][9*Cin] with the tap (ty*3+tx) major and the input channel minor,
// padded with zeros to a multiple of 16.
//
// Forward, level l with 16 or more output channels: im2col of the upsampled
// input (k_im2col_up, never materialising the upsampled grid) and the
// tensor-core product (im2col x W^T, bias and ReLU in the epilogue).  A level
// with fewer output channels (the map's one, or 8) is below the tensor
// cores' narrowest tile and runs as a direct convolution (k_dec_conv).
// Backward: the output gradient in BF16 (k_to_bf16); the weight and bias
// gradients by k_dec_dw (per chunk of pixels, FP32 sums of BF16 products
// read straight from the level input, then summed over the chunks); the
// input gradient by k_dec_dx (FP32 sums of BF16 products over the taps and
// the 2x2 upsampled cells).  The direct kernels keep the weights in shared
// memory as FP32, [tap][input channel][output channel], with CO >= Cout
// output channels (zeros past Cout), and every sum runs in a fixed order, so
// training is deterministic.
#pragma once
#include <cuda_bf16.h>

#include <cstdint>

namespace cliffs_nn {

// im2col of the 2x upsampled input: row p = (b, Y, X) of the output grid
// (side 2S), column k = tap * Cin + c < 9 Cin, columns up to kp zero.  The
// upsampled cell (Y', X') = (Y + ty - 1, X + tx - 1) reads input cell
// (Y' / 2, X' / 2); outside [0, 2S) it is zero padding.  dst [P][kp].  Block
// (32, 8): eight pixels, each thread 8 columns at a time (one tap, 8
// channels: C and kp are multiples of 8), one 16-byte load and store.  Pixel
// indices are 32-bit (B (2S)^2 < 2^31).
__global__ void k_im2col_up(int B, int S, int C, const __nv_bfloat16* __restrict__ x, int kp, __nv_bfloat16* dst) {
  const int S2 = 2 * S, img = S2 * S2;
  const int p = blockIdx.x * 8 + threadIdx.y;
  if (p >= B * img) return;
  const int b = p / img, r = p % img, Y = r / S2, X = r % S2;
  uint4* out = reinterpret_cast<uint4*>(dst + (size_t)p * kp);
  for (int kq = threadIdx.x; kq < kp / 8; kq += 32) {
    const int k = 8 * kq;
    uint4 v = make_uint4(0u, 0u, 0u, 0u);
    if (k < 9 * C) {
      const int tap = k / C, c = k % C;
      const int Yu = Y + tap / 3 - 1, Xu = X + tap % 3 - 1;
      if (Yu >= 0 && Yu < S2 && Xu >= 0 && Xu < S2)
        v = __ldg(reinterpret_cast<const uint4*>(x + (((size_t)b * S + (Yu >> 1)) * S + (Xu >> 1)) * C + c));
    }
    out[kq] = v;
  }
}

// The decoder's input: ReLU of the latent columns [col0, col0 + n) of the
// dense output (rows of ld floats) in BF16.
__global__ void k_dec_input(int B, int n, const float* __restrict__ y, int ld, int col0, __nv_bfloat16* x) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= B * n) return;
  const int b = t / n, j = t % n;
  x[t] = __float2bfloat16(fmaxf(y[(size_t)b * ld + col0 + j], 0.f));
}

// Squared-error loss of one output block: y rows (ld_y floats, from column
// y0) against target rows idx[r] (or r) of tg (ld_t floats, from column t0),
// n values per row.  dy (ld_d floats per row, from column d0) gets
// scale (y - t); part[blockIdx.x] a partial sum of (y - t)^2 in a fixed order.
__global__ void __launch_bounds__(256) k_mse_block(int B, int n, const float* __restrict__ y, int ld_y, int y0,
                                                   const float* __restrict__ tg, int ld_t, int t0,
                                                   const int* __restrict__ idx, float* dy, int ld_d, int d0,
                                                   float scale, float* part) {
  __shared__ float s[256];
  float acc = 0.f;
  const int total = B * n;  // < 2^31
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < total; k += gridDim.x * blockDim.x) {
    const int r = k / n, j = k % n;
    const int tr = idx ? idx[r] : r;
    const float d = y[(size_t)r * ld_y + y0 + j] - tg[(size_t)tr * ld_t + t0 + j];
    dy[(size_t)r * ld_d + d0 + j] = scale * d;
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

// Partial sums [splits][rows][ldp] summed into out [rows][cols] (cols <=
// ldp): block (32 outputs) x (kStrands strands); strand s adds the splits
// z = s, s + kStrands, ... in order, and the strand sums are added in strand
// order, so the result does not depend on the launch.  Column sums of a
// matrix [R][N] are the case rows = 1, cols = ldp = N, splits = R.
constexpr int kStrands = 16;
__global__ void __launch_bounds__(32 * kStrands) k_reduce_wgrad(int rows, int cols, int ldp, int splits,
                                                               const float* __restrict__ part, float* out) {
  __shared__ float sh[kStrands][33];
  const int lane = threadIdx.x & 31, strand = threadIdx.x >> 5;
  const int k = blockIdx.x * 32 + lane;
  const bool in = k < rows * cols;
  float s = 0.f;
  if (in) {
    const int r = k / cols, c = k % cols;
    for (int z = strand; z < splits; z += kStrands) s += part[((size_t)z * rows + r) * ldp + c];
  }
  sh[strand][lane] = s;
  __syncthreads();
  if (strand == 0 && in) {
    float t = 0.f;
#pragma unroll
    for (int i = 0; i < kStrands; ++i) t += sh[i][lane];
    out[k] = t;
  }
}

// FP32 to BF16, n values.
__global__ void k_to_bf16(int n, const float* __restrict__ src, __nv_bfloat16* dst) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) dst[t] = __float2bfloat16(src[t]);
}

// Input channels per thread of the direct kernels: G x CO FP32 sums.
template <int CO>
__host__ __device__ constexpr int dec_group() {
  return CO == 1 ? 8 : CO == 8 ? 4 : CO == 16 ? 2 : 1;
}

// The 8 BF16 values of a 16-byte load as FP32.
__device__ __forceinline__ void unpack8(const uint4 q, float (&v)[8]) {
  const uint32_t w[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    v[2 * i] = __uint_as_float(w[i] << 16);
    v[2 * i + 1] = __uint_as_float(w[i] & 0xffff0000u);
  }
}

// G consecutive BF16 values (G = 1, 2, 4 or 8; 2G-byte aligned) as FP32.
template <int G>
__device__ __forceinline__ void load_bf16(const __nv_bfloat16* p, float (&v)[G]) {
  if constexpr (G == 8) {
    float t[8];
    unpack8(__ldg(reinterpret_cast<const uint4*>(p)), t);
#pragma unroll
    for (int i = 0; i < 8; ++i) v[i] = t[i];
  } else if constexpr (G == 4) {
    const uint2 q = __ldg(reinterpret_cast<const uint2*>(p));
    v[0] = __uint_as_float(q.x << 16);
    v[1] = __uint_as_float(q.x & 0xffff0000u);
    v[2] = __uint_as_float(q.y << 16);
    v[3] = __uint_as_float(q.y & 0xffff0000u);
  } else if constexpr (G == 2) {
    const uint32_t q = __ldg(reinterpret_cast<const unsigned int*>(p));
    v[0] = __uint_as_float(q << 16);
    v[1] = __uint_as_float(q & 0xffff0000u);
  } else {
    v[0] = __bfloat162float(p[0]);
  }
}

// The weights w [co][kp] (BF16, columns k = tap * C + c) into shared memory
// as FP32 [9C][CO], zero past co.  The whole block calls it.
template <int CO>
__device__ __forceinline__ void stage_weights(float* sw, int C, int co, const __nv_bfloat16* __restrict__ w, int kp) {
  const int K = 9 * C;
  for (int t = threadIdx.x; t < K * CO; t += blockDim.x) {
    const int k = t / CO, o = t % CO;
    sw[t] = o < co ? __bfloat162float(w[(size_t)o * kp + k]) : 0.f;
  }
  __syncthreads();
}

// Direct forward convolution of a level with co <= CO output channels (CO =
// 1 or 8): one thread per output pixel p = (b, Y, X) of the 2S x 2S grid,
// FP32 sums over the taps (in order) and the input channels, bias added;
// then either ReLU and a BF16 row of co values (out16, NHWC) or the FP32
// value of the one-channel map (out32).  C a multiple of 8.  Dynamic shared
// memory: 9 C CO floats.
template <int CO>
__global__ void __launch_bounds__(256) k_dec_conv(int B, int S, int C, int co, const __nv_bfloat16* __restrict__ x,
                                                  const __nv_bfloat16* __restrict__ w, int kp,
                                                  const float* __restrict__ bias, __nv_bfloat16* out16, float* out32) {
  extern __shared__ float sw[];
  stage_weights<CO>(sw, C, co, w, kp);
  const int S2 = 2 * S, img = S2 * S2;
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= B * img) return;
  const int b = p / img, r = p % img;
  const int Y = r / S2, X = r % S2;
  float acc[CO];
#pragma unroll
  for (int o = 0; o < CO; ++o) acc[o] = 0.f;
  for (int tap = 0; tap < 9; ++tap) {
    const int Yu = Y + tap / 3 - 1, Xu = X + tap % 3 - 1;
    if (Yu < 0 || Yu >= S2 || Xu < 0 || Xu >= S2) continue;
    const __nv_bfloat16* xr = x + (((size_t)b * S + (Yu >> 1)) * S + (Xu >> 1)) * C;
    const float* wt = sw + tap * C * CO;
    for (int c8 = 0; c8 < C; c8 += 8) {
      float xv[8];
      load_bf16<8>(xr + c8, xv);
#pragma unroll
      for (int g = 0; g < 8; ++g)
#pragma unroll
        for (int o = 0; o < CO; ++o) acc[o] = fmaf(xv[g], wt[(c8 + g) * CO + o], acc[o]);
    }
  }
  if (out16) {
#pragma unroll
    for (int o = 0; o < CO; ++o)
      if (o < co) out16[(size_t)p * co + o] = __float2bfloat16(fmaxf(acc[o] + bias[o], 0.f));
  } else {
    out32[p] = acc[0] + bias[0];
  }
}

// Partial weight and bias gradients of a level over one chunk of output
// pixels (block z: pixels [z chunk, (z+1) chunk)).  dW[o][k] is the sum over
// pixels p of dz[p][o] times the im2col value of column k = tap * C + c at p,
// read from the level input x (B, S, S, C) through the 2x upsampling and the
// zero padding; db[o] the sum of dz[p][o].  The 9C/G groups of G input
// channels of one tap are spread over blockIdx.y, KGb = min(9C/G, blockDim)
// groups per block; thread (slot s, group kg) owns the G channels
// c0 = (kg % (C/G)) G .. of tap kg / (C/G) and all CO outputs, and takes
// every NS-th pixel of each staged run of kStage pixels (NS = blockDim / KGb
// slots); the slots' sums are then added in slot order.  dz holds BF16 rows
// of ldz values (co used).  part [blocks][co][9C], part_b [blocks][co]
// (from blockIdx.y = 0).  Dynamic shared memory: dec_dw_smem<CO>(C) bytes.
constexpr int kStage = 128;
template <int CO>
__host__ __device__ constexpr size_t dec_dw_smem(int C) {
  return (size_t)kStage * CO * 4 + (size_t)kStage * 8 + (size_t)9 * C * CO * 4;
}
template <int CO>
__global__ void __launch_bounds__(256) k_dec_dw(int B, int S, int C, int co, const __nv_bfloat16* __restrict__ dz,
                                                int ldz, const __nv_bfloat16* __restrict__ x, int chunk,
                                                float* part, float* part_b) {
  constexpr int G = dec_group<CO>();
  extern __shared__ float sm[];
  float* sdz = sm;                                          // [kStage][CO]
  int2* spix = reinterpret_cast<int2*>(sdz + kStage * CO);  // (b S, Y << 16 | X); Y = -1 past the end
  float* sacc = reinterpret_cast<float*>(spix + kStage);    // [9C][CO]
  const int K = 9 * C, KG = K / G, KGb = min(KG, (int)blockDim.x), NS = (int)blockDim.x / KGb;
  const int t = threadIdx.x;
  const int kg = (int)blockIdx.y * KGb + t % KGb, slot = t / KGb;
  const bool worker = slot < NS && kg < KG;
  const int tap = kg / (C / G), c0 = (kg % (C / G)) * G;
  const int dy = tap / 3 - 1, dxo = tap % 3 - 1;
  const int S2 = 2 * S, img = S2 * S2, P = B * img;
  const int p0 = blockIdx.x * chunk;
  float acc[G][CO];
#pragma unroll
  for (int g = 0; g < G; ++g)
#pragma unroll
    for (int o = 0; o < CO; ++o) acc[g][o] = 0.f;
  float bsum = 0.f;
  for (int r0 = 0; r0 < chunk; r0 += kStage) {
    __syncthreads();  // the previous run is consumed
    for (int i = t; i < kStage * CO; i += blockDim.x) {
      const int j = i / CO, o = i % CO;
      const int p = p0 + r0 + j;
      sdz[i] = (r0 + j < chunk && p < P && o < co) ? __bfloat162float(dz[(size_t)p * ldz + o]) : 0.f;
    }
    for (int j = t; j < kStage; j += blockDim.x) {
      const int p = p0 + r0 + j;
      int2 v = make_int2(0, -4 * 65536);  // row -4: every tap outside the grid
      if (r0 + j < chunk && p < P) {
        const int b = p / img, r = p % img;
        v = make_int2(b * S, (r / S2) << 16 | (r % S2));
      }
      spix[j] = v;
    }
    __syncthreads();
    if (t < co)
      for (int j = 0; j < kStage; ++j) bsum += sdz[j * CO + t];
    if (worker) {
      for (int j = slot; j < kStage; j += NS) {
        const int2 v = spix[j];
        const int Yu = (v.y >> 16) + dy, Xu = (v.y & 0xffff) + dxo;
        if (Yu < 0 || Yu >= S2 || Xu < 0 || Xu >= S2) continue;
        float xv[G];
        load_bf16<G>(x + ((size_t)(v.x + (Yu >> 1)) * S + (Xu >> 1)) * C + c0, xv);
        const float* d = sdz + j * CO;
#pragma unroll
        for (int o = 0; o < CO; ++o) {
          const float dv = d[o];
#pragma unroll
          for (int g = 0; g < G; ++g) acc[g][o] = fmaf(dv, xv[g], acc[g][o]);
        }
      }
    }
  }
  // the slots' sums, added in slot order
  for (int i = t; i < K * CO; i += blockDim.x) sacc[i] = 0.f;
  for (int s = 0; s < NS; ++s) {
    __syncthreads();
    if (worker && slot == s)
#pragma unroll
      for (int g = 0; g < G; ++g)
#pragma unroll
        for (int o = 0; o < CO; ++o) sacc[(kg * G + g) * CO + o] += acc[g][o];
  }
  __syncthreads();
  const int kb = (int)blockIdx.y * KGb * G, kn = min(K - kb, KGb * G);  // this block's columns
  for (int i = t; i < co * kn; i += blockDim.x) {
    const int o = i / kn, k = kb + i % kn;
    part[((size_t)blockIdx.x * co + o) * K + k] = sacc[k * CO + o];
  }
  if (blockIdx.y == 0 && t < co) part_b[(size_t)blockIdx.x * co + t] = bsum;
}

// Gradient of the level input x (B, S, S, C) from the output gradient dz
// (B, 2S, 2S pixels of ldz BF16 values, co used) and the weights w [co][kp]:
// the 3x3 correlation transposed, summed over the 2x2 cells each input cell
// was copied to.  One thread per input cell and group of G channels, the
// cell varying fastest (a warp reads the same weights), FP32 sums in a fixed
// order.  dz rows of ldz values are 16-byte aligned when co > 1 (co a
// multiple of 8).  mask (optional): x's own values, the ReLU derivative
// applied (x > 0).  Sample b's S*S*C values go to dx + b * ld + col0.
// Dynamic shared memory: 9 C CO floats.
template <int CO>
__global__ void __launch_bounds__(256) k_dec_dx(int B, int S, int C, int co, const __nv_bfloat16* __restrict__ dz,
                                                int ldz, const __nv_bfloat16* __restrict__ w, int kp,
                                                const __nv_bfloat16* __restrict__ mask, float* dx, int ld,
                                                int col0) {
  constexpr int G = dec_group<CO>();
  extern __shared__ float sw[];
  stage_weights<CO>(sw, C, co, w, kp);
  const int ncell = B * S * S;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ncell * (C / G)) return;
  const int c0 = (t / ncell) * G;
  const int q = t % ncell;  // input cell
  const int x0 = q % S, y0 = (q / S) % S, b = q / (S * S);
  const int S2 = 2 * S;
  const int nq = co / 8;  // 16-byte loads of a dz row (co > 1)
  float acc[G];
#pragma unroll
  for (int g = 0; g < G; ++g) acc[g] = 0.f;
  for (int a = 0; a < 2; ++a)
    for (int e = 0; e < 2; ++e) {
      const int Yu = 2 * y0 + a, Xu = 2 * x0 + e;  // the upsampled cell
      for (int ty = 0; ty < 3; ++ty) {
        const int Y = Yu - (ty - 1);  // output row that read (Yu, Xu) through tap ty
        if (Y < 0 || Y >= S2) continue;
        for (int tx = 0; tx < 3; ++tx) {
          const int X = Xu - (tx - 1);
          if (X < 0 || X >= S2) continue;
          const __nv_bfloat16* g = dz + (((size_t)b * S2 + Y) * S2 + X) * ldz;
          float dv[CO];
          if constexpr (CO == 1) {
            dv[0] = __bfloat162float(g[0]);
          } else {
#pragma unroll
            for (int i = 0; i < CO / 8; ++i) {
              float t8[8];
              if (i < nq) {
                unpack8(__ldg(reinterpret_cast<const uint4*>(g) + i), t8);
              } else {
#pragma unroll
                for (int h = 0; h < 8; ++h) t8[h] = 0.f;
              }
#pragma unroll
              for (int h = 0; h < 8; ++h) dv[8 * i + h] = t8[h];
            }
          }
          const float* wt = sw + ((ty * 3 + tx) * C + c0) * CO;
#pragma unroll
          for (int gg = 0; gg < G; ++gg)
#pragma unroll
            for (int o = 0; o < CO; ++o) acc[gg] = fmaf(dv[o], wt[gg * CO + o], acc[gg]);
        }
      }
    }
  const size_t i0 = (size_t)q * C + c0;  // index of the first channel in x
  float* out = dx + (size_t)b * ld + col0 + (i0 - (size_t)b * S * S * C);
#pragma unroll
  for (int gg = 0; gg < G; ++gg) {
    float v = acc[gg];
    if (mask && !(__bfloat162float(mask[i0 + gg]) > 0.f)) v = 0.f;
    out[gg] = v;
  }
}

}  // namespace cliffs_nn
