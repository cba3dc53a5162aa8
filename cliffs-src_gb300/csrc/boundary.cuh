// boundary.cuh -- ComputeBoundaryInput (cmpboundary/cmpboundary.f:44-190) on
// the device: the edge forcing of a target grid from a coarse sea-state cube
// (the feed get_boundary_feed.f reads).
//
// The host cuts the cube down to the target's footprint in the source
// lattice: columns W_nx .. E_nx+1, rows S_ny .. N_ny+1, records from the
// first signal on.  Then:
//   k_boundary_scan   scan4wave.f: per record, the largest value and the
//                     largest negated value over the footprint, missing
//                     values (below -1e10) as 0; a block per record.
//   k_boundary_edges  InterpolateOntoBndr.f:6-38: each edge node's value,
//                     linear across the edge between the two lattice
//                     columns (rows) that straddle it, then linear along the
//                     edge; a thread per edge node and record.
// The products and sums are rounded one by one (no fused multiply-add), as
// the CPU restatement does, so the records are bit-identical to it.
#pragma once

namespace cliffs {

__device__ __forceinline__ double sea_value(const float* sea, int nx, int ny, int i, int j, int k, float scale) {
  float v = sea[(size_t)(i - 1) + (size_t)(j - 1) * nx + (size_t)(k - 1) * nx * ny];
  if (v < -1.0e10f) v = 0.0f;                 // where(sea < nanum) sea = 0
  if (scale != 1.0f) v = __fmul_rn(v, scale);  // sea = 0.01*sea, a real*4 product
  return (double)v;
}

// a*x + (1-a)*y, rounded step by step
__device__ __forceinline__ double mix(double a, double x, double y) {
  return __dadd_rn(__dmul_rn(a, x), __dmul_rn(__dadd_rn(1.0, -a), y));
}

__global__ void k_boundary_scan(int nx, int ny, const float* __restrict__ sea, float* __restrict__ hi,
                                float* __restrict__ lo) {
  const size_t n = (size_t)nx * ny;
  const float* s = sea + (size_t)blockIdx.x * n;
  float mx = -INFINITY, mn = -INFINITY;
  for (size_t k = threadIdx.x; k < n; k += blockDim.x) {
    float v = s[k];
    if (v < -1.0e10f) v = 0.0f;
    mx = fmaxf(mx, v);
    mn = fmaxf(mn, -v);
  }
  __shared__ float smx[32], smn[32];
  for (int o = 16; o > 0; o >>= 1) {
    mx = fmaxf(mx, __shfl_down_sync(0xffffffffu, mx, o));
    mn = fmaxf(mn, __shfl_down_sync(0xffffffffu, mn, o));
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) {
    smx[warp] = mx;
    smn[warp] = mn;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) {
      mx = fmaxf(mx, smx[w]);
      mn = fmaxf(mn, smn[w]);
    }
    hi[blockIdx.x] = mx;
    lo[blockIdx.x] = mn;
  }
}

// Component ival (1 u, 2 v, 3 eta) of west/east [nt][3][nn] and
// south/north [nt][3][mm].  Tables as cliffs_nest_desc, device copies of the
// per-node arrays.
__global__ void k_boundary_edges(int nx, int ny, int nt, const float* __restrict__ sea, float scale, int ival,
                                 int mm, int nn, double W_cx, double E_cx, double S_cy, double N_cy,
                                 const int32_t* __restrict__ WE_ny, const double* __restrict__ WE_cy,
                                 const int32_t* __restrict__ SN_nx, const double* __restrict__ SN_cx, double* west,
                                 double* east, double* south, double* north) {
  const int per = nn + mm;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)per * nt) return;
  const int k = (int)(t / per) + 1, node = (int)(t % per);
  if (node < nn) {
    const int i = node + 1;
    const int kk = WE_ny[i - 1] - WE_ny[0] + 1;
    const double cc = WE_cy[i - 1];
    const double w1 = mix(W_cx, sea_value(sea, nx, ny, 1, kk, k, scale), sea_value(sea, nx, ny, 2, kk, k, scale));
    const double w2 =
        mix(W_cx, sea_value(sea, nx, ny, 1, kk + 1, k, scale), sea_value(sea, nx, ny, 2, kk + 1, k, scale));
    const double e1 =
        mix(E_cx, sea_value(sea, nx, ny, nx - 1, kk, k, scale), sea_value(sea, nx, ny, nx, kk, k, scale));
    const double e2 =
        mix(E_cx, sea_value(sea, nx, ny, nx - 1, kk + 1, k, scale), sea_value(sea, nx, ny, nx, kk + 1, k, scale));
    const size_t o = (size_t)(i - 1) + (size_t)(ival - 1) * nn + (size_t)(k - 1) * 3 * nn;
    west[o] = mix(cc, w1, w2);
    east[o] = mix(cc, e1, e2);
  } else {
    const int i = node - nn + 1;
    const int kk = SN_nx[i - 1] - SN_nx[0] + 1;
    const double cc = SN_cx[i - 1];
    const double s1 = mix(S_cy, sea_value(sea, nx, ny, kk, 1, k, scale), sea_value(sea, nx, ny, kk, 2, k, scale));
    const double s2 =
        mix(S_cy, sea_value(sea, nx, ny, kk + 1, 1, k, scale), sea_value(sea, nx, ny, kk + 1, 2, k, scale));
    const double n1 =
        mix(N_cy, sea_value(sea, nx, ny, kk, ny - 1, k, scale), sea_value(sea, nx, ny, kk, ny, k, scale));
    const double n2 =
        mix(N_cy, sea_value(sea, nx, ny, kk + 1, ny - 1, k, scale), sea_value(sea, nx, ny, kk + 1, ny, k, scale));
    const size_t o = (size_t)(i - 1) + (size_t)(ival - 1) * mm + (size_t)(k - 1) * 3 * mm;
    south[o] = mix(cc, s1, s2);
    north[o] = mix(cc, n1, n2);
  }
}

}  // namespace cliffs
