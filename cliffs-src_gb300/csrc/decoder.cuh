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
// Forward, level l: im2col of the upsampled input (k_im2col_up, never
// materialising the upsampled grid) and the tensor-core product gemm_tn
// (im2col x W^T, bias and ReLU in the epilogue).  Backward: the output
// gradient in BF16 (k_pack_grad), the weight gradient as a split-K product
// dZ^T x im2col summed over the splits in a fixed order, the bias gradient as
// a two-stage column sum, and the input gradient by k_dec_dx (FP32 sums of
// BF16 products over the taps and the 2x2 upsampled cells).  Every sum runs
// in a fixed order, so training is deterministic.
#pragma once
#include <cuda_bf16.h>

namespace cliffs_nn {

// im2col of the 2x upsampled input: row p = (b, Y, X) of the output grid
// (side 2S), column k = tap * Cin + c < 9 Cin, columns up to kp zero.  The
// upsampled cell (Y', X') = (Y + ty - 1, X + tx - 1) reads input cell
// (Y' / 2, X' / 2); outside [0, 2S) it is zero padding.  dst [P][kp], and
// dst_t [kp][ldt] (transposed) when given.
__global__ void k_im2col_up(int B, int S, int C, const __nv_bfloat16* __restrict__ x, int kp, __nv_bfloat16* dst,
                            __nv_bfloat16* dst_t, int ldt) {
  const int S2 = 2 * S;
  const long long P = (long long)B * S2 * S2;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= P * kp) return;
  const long long p = t / kp;
  const int k = (int)(t % kp);
  __nv_bfloat16 v = __float2bfloat16(0.f);
  if (k < 9 * C) {
    const int tap = k / C, c = k % C;
    const int b = (int)(p / ((long long)S2 * S2));
    const int r = (int)(p % ((long long)S2 * S2));
    const int Y = r / S2 + tap / 3 - 1, X = r % S2 + tap % 3 - 1;
    if (Y >= 0 && Y < S2 && X >= 0 && X < S2) v = x[(((size_t)b * S + (Y >> 1)) * S + (X >> 1)) * C + c];
  }
  dst[(size_t)p * kp + k] = v;
  if (dst_t) dst_t[(size_t)k * ldt + p] = v;
}

// The decoder's input: ReLU of the latent columns [col0, col0 + n) of the
// dense output (rows of ld floats) in BF16.
__global__ void k_dec_input(int B, int n, const float* __restrict__ y, int ld, int col0, __nv_bfloat16* x) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)B * n) return;
  const int b = (int)(t / n), j = (int)(t % n);
  x[t] = __float2bfloat16(fmaxf(y[(size_t)b * ld + col0 + j], 0.f));
}

// Gradient of the level input x (B, S, S, C) from the output gradient dz
// (B, 2S, 2S pixels of ldz values, the first Co used) in BF16 and the
// weights w [Co][kp]: the 3x3 correlation transposed, summed over the 2x2
// cells each input cell was copied to.  mask (optional): x's own values, the
// ReLU derivative applied (x > 0).  Sample b's S*S*C values go to
// dx + b * ld + col0.
__global__ void k_dec_dx(int B, int S, int C, int Co, const __nv_bfloat16* __restrict__ dz, int ldz,
                         const __nv_bfloat16* __restrict__ w, int kp, const __nv_bfloat16* __restrict__ mask,
                         float* dx, int ld, int col0) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)B * S * S * C) return;
  const int c = (int)(t % C);
  const long long q = t / C;
  const int x0 = (int)(q % S), y0 = (int)((q / S) % S), b = (int)(q / ((long long)S * S));
  const int S2 = 2 * S;
  float acc = 0.f;
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
          const __nv_bfloat16* wk = w + (ty * 3 + tx) * C + c;
          for (int o = 0; o < Co; ++o) acc += __bfloat162float(g[o]) * __bfloat162float(wk[(size_t)o * kp]);
        }
      }
    }
  if (mask && !(__bfloat162float(mask[t]) > 0.f)) acc = 0.f;
  const long long per = (long long)S * S * C;
  dx[(size_t)b * ld + col0 + (size_t)(t - (long long)b * per)] = acc;
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
  const long long total = (long long)B * n;
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < total;
       k += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(k / n), j = (int)(k % n);
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

// The split partials [splits][rows][ldp] of a weight gradient summed in split
// order into out [rows][cols] (cols <= ldp).
__global__ void k_reduce_wgrad(int rows, int cols, int ldp, int splits, const float* __restrict__ part,
                               float* out) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= rows * cols) return;
  const int r = k / cols, c = k % cols;
  float s = 0.f;
  for (int z = 0; z < splits; ++z) s += part[((size_t)z * rows + r) * ldp + c];
  out[k] = s;
}

// A level's FP32 output gradient dz [P][N] into BF16 rows dzb [P][cp] (zero
// past N) and the transpose dzt [N][P].
__global__ void k_pack_grad(long long P, int N, int cp, const float* __restrict__ dz, __nv_bfloat16* dzb,
                            __nv_bfloat16* dzt) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= P * cp) return;
  const long long r = t / cp;
  const int c = (int)(t % cp);
  const float v = c < N ? dz[(size_t)r * N + c] : 0.f;
  const __nv_bfloat16 h = __float2bfloat16(v);
  dzb[t] = h;
  if (c < N) dzt[(size_t)c * P + r] = h;
}

// Sum of `splits` partial [n] arrays into out, in split order.
__global__ void k_reduce_splits(int n, int splits, const float* __restrict__ part, float* out) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  float s = 0.f;
  for (int z = 0; z < splits; ++z) s += part[(size_t)z * n + k];
  out[k] = s;
}

// Column sums of dy [R][N] in two stages: block (c, z) sums rows z*chunk ..
// in order into part[z][c]; then k_reduce_splits.
__global__ void k_colsum_part(int R, int N, int chunk, const float* __restrict__ dy, float* part) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= N) return;
  const long long r0 = (long long)blockIdx.y * chunk;
  const long long r1 = min((long long)R, r0 + chunk);
  float s = 0.f;
  for (long long r = r0; r < r1; ++r) s += dy[(size_t)r * N + c];
  part[(size_t)blockIdx.y * N + c] = s;
}

}  // namespace cliffs_nn
