// ytile.cuh -- the y-sweep of a two-dimensional step with its tile staged in
// shared memory by the bulk-copy (TMA) engine, in and out.
//
// fast_kernel's y-sweep loads its window with 24 scalar loads a thread (6
// rows of 4 fields, lanes along the row) and stores 12 scalars, each with its
// own 64-bit address: per cell it issues twice the integer and memory
// instructions of the x-sweep, whose rows move as float4s.  Here a block owns
// the tile of 16 rows x 32 columns of fast_kernel's y blocks (4 warps, a warp
// per 4 rows, a lane per column).  One thread issues the four 2-D tensor-map
// copies of the window (32 columns x 18 rows: the tile and one halo row on
// each side; rows outside the grid read 0), every thread reads its 6-cell
// window from shared memory at fixed offsets, computes its 4 cells with
// sweep_cells (the arithmetic of fast_kernel, so the results are the same
// bits), and writes them into an output tile in shared memory.  The block's
// listed cells (shorelines, line ends) are finished into the same tile, and
// one thread stores the three output fields with three tensor-map copies,
// which clip rows and columns outside the grid.
//
// A row outside the grid reads 0 where fast_kernel reads a copy of the line's
// end cell: such a window cell never enters a cell that is kept, as the plain
// update needs 2 <= k <= n-1 and the line-end rules use cells 1..n only.
//
// Bands are taken last to first as in fast_kernel's y grid (the rows the
// x-sweep wrote last are still in L2).  The wait for the window copies is
// bounded (StageCtl::wait_ns); a block whose wait runs out records ST_STALL,
// waits (bounded) for its copies once more and leaves without storing.
//
// batch_tile_y runs the same body for the y phase of a batched step (one
// tile per list entry of batch.cuh), with each scenario's tensor maps in
// device memory.
#pragma once
#include "batch.cuh"
#include "staged.cuh"

namespace cliffs {

static_assert(kYRows * 32 == kYTileCells, "a y tile is 16 rows of 32 columns");

// Tensor maps of one y-sweep: the input copy's fields with a 32 x kYWin box
// (loads), the output copy's with a 32 x kYRows box (stores).
struct YTileMaps {
  CUtensorMap dep, srf, xu, yv;
  CUtensorMap srf_o, xu_o, yv_o;
};

// 9 blocks per SM (56 registers, 16 bytes of spills): each block waits for
// its tile's copies before it computes, and the ninth block hides more of
// that wait than the eighth's registers would save (per-sweep event time
// 30.8 against 31.6 us on the 2048^2 shelf; 48 registers: 32.3 us).
template <bool FLAT>
__global__ void __launch_bounds__(128, 9)
    tile_y_kernel(const SweepArgs A, const __grid_constant__ YTileMaps M, const StageCtl S) {
  __shared__ __align__(128) float s_in[4][kYWin][32];  // dep, srf, xu, yv; row + 1 - r0, col - c0
  __shared__ __align__(128) float s_out[3][kYRows][32];  // srf, xu, yv; row - r0, col - c0
  __shared__ uint32_t s_list[kYTileCells];
  __shared__ unsigned s_n;
  __shared__ __align__(8) uint64_t bar;
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int c0 = (int)blockIdx.x * 32;                             // first column (0-based)
  const int r0 = (int)(gridDim.y - 1 - blockIdx.y) * kYRows;       // first row (0-based)
  if (tid == 0) {
    mbar_init(&bar, 1);
    s_n = 0u;
    fence_mbar_init();
  }
  __syncthreads();
  // every thread: the previous grid complete, its stores visible
  asm volatile("griddepcontrol.wait;" ::: "memory");
  constexpr uint32_t kWinBytes = kYWin * 32 * 4;
  if (tid == 0) {
    mbar_expect_tx(&bar, 4u * kWinBytes + S.extra);
    tma_load_2d(&s_in[0][0][0], &M.dep, &bar, c0, r0 - 1);
    tma_load_2d(&s_in[1][0][0], &M.srf, &bar, c0, r0 - 1);
    tma_load_2d(&s_in[2][0][0], &M.xu, &bar, c0, r0 - 1);
    tma_load_2d(&s_in[3][0][0], &M.yv, &bar, c0, r0 - 1);
  }
  const bool ok = mbar_wait_ns(&bar, 0u, S.wait_ns);
  if (__syncthreads_or(!ok)) {
    if (tid == 0) {
      atomicOr(A.status, ST_STALL);
      mbar_wait_ns(&bar, 0u, S.wait_ns);  // the copies in flight, before the block's memory goes
    }
    return;
  }
  const int L = c0 + lane + 1;
  const int i0 = r0 + warp * kCellsPerThread + 1;
  const bool active = L <= A.nlines && i0 <= A.n;
  float d[6], e[6], u[6], v[6];
  float hm[kCellsPerThread], vm[kCellsPerThread];
#pragma unroll
  for (int w = 0; w < 6; ++w) {
    const int r = warp * kCellsPerThread + w;
    d[w] = s_in[0][r][lane];
    e[w] = s_in[1][r][lane];
    v[w] = s_in[2][r][lane];  // tangential in the y-sweep
    u[w] = s_in[3][r][lane];  // normal
  }
#pragma unroll
  for (int r = 0; r < kCellsPerThread; ++r) {
    hm[r] = vm[r] = 0.f;
    if (!active) {
      // columns past the grid hold 0, as the row padding does: the tile
      // store may write the padding of a row's last 16 bytes
      s_out[0][warp * kCellsPerThread + r][lane] = 0.f;
      s_out[1][warp * kCellsPerThread + r][lane] = 0.f;
      s_out[2][warp * kCellsPerThread + r][lane] = 0.f;
    }
  }
  sweep_cells<1, true, false, false, false, false, FLAT, true>(A, L, i0, active, 0, d, e, u, v, hm, vm, s_list,
                                                               &s_n,
                                                               &s_out[0][warp * kCellsPerThread][lane]);
  __syncthreads();  // the fast values are in the tile; the listed cells overwrite theirs
  const unsigned cnt = s_n;
  bool bad = false;
  for (unsigned t = tid; t < cnt; t += blockDim.x) bad |= !general_to_tile<false>(A, s_list[t], &s_out[0][0][0], r0, c0);
  if (bad) atomicOr(A.status, ST_NAN);
  fence_proxy_async_smem();  // this thread's tile writes, before the copy engine reads them
  __syncthreads();
  if (tid == 0) {
    tma_store_2d(&M.srf_o, &s_out[0][0][0], c0, r0);
    tma_store_2d(&M.xu_o, &s_out[1][0][0], c0, r0);
    tma_store_2d(&M.yv_o, &s_out[2][0][0], c0, r0);
    bulk_commit();
    bulk_wait_read();  // the tile stays until the copies have read it
  }
}

// The y phase of a batched step (one launch for every scenario's y tiles,
// one tile per block): tile_y_kernel's body on the scenario that the list
// entry names, with the scenario's arguments staged in shared memory and its
// tensor maps read from B.ymaps (device memory, written before the launch).
// FLAT: every scenario flat along y.
template <bool FLAT>
__global__ void __launch_bounds__(128, 9) batch_tile_y(const BatchArgs B) {
  __shared__ SweepArgs sA;
  __shared__ __align__(128) float s_in[4][kYWin][32];
  __shared__ __align__(128) float s_out[3][kYRows][32];
  __shared__ uint32_t s_list[kYTileCells];
  __shared__ unsigned s_n;
  __shared__ __align__(8) uint64_t bar;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int* off = B.off + (B.n + 1);
  const int t = blockIdx.x;
  const int k = batch_scenario(off, B.n, t);
  const int local = t - __ldg(off + k);
  const int g = __ldg(B.gx + B.n + k);  // row groups of the scenario
  const int r0 = (local % g) * kYRows, c0 = (local / g) * 32;
  const YTileMaps* M = B.ymaps + k;
  constexpr uint32_t kWinBytes = kYWin * 32 * 4;
  if (tid == 0) {
    mbar_init(&bar, 1);
    s_n = 0u;
    fence_mbar_init();
    // B.extra (the timeout self-test): 16 bytes more than the copies bring
    mbar_expect_tx(&bar, 4u * kWinBytes + (B.extra ? 16u : 0u));
    tma_load_2d(&s_in[0][0][0], &M->dep, &bar, c0, r0 - 1);
    tma_load_2d(&s_in[1][0][0], &M->srf, &bar, c0, r0 - 1);
    tma_load_2d(&s_in[2][0][0], &M->xu, &bar, c0, r0 - 1);
    tma_load_2d(&s_in[3][0][0], &M->yv, &bar, c0, r0 - 1);
    sA = B.args[2 * k + 1];
  }
  __syncthreads();
  const bool ok = mbar_wait_ns(&bar, 0u, B.wait_ns);
  if (__syncthreads_or(!ok)) {
    if (tid == 0) {
      atomicOr(sA.status, ST_STALL);
      atomicOr(B.err, 1u);
      mbar_wait_ns(&bar, 0u, B.wait_ns);  // the copies in flight, before the block's memory goes
    }
    return;
  }
  const int L = c0 + lane + 1;
  const int i0 = r0 + warp * kCellsPerThread + 1;
  const bool active = L <= sA.nlines && i0 <= sA.n;
  float d[6], e[6], u[6], v[6];
  float hm[kCellsPerThread], vm[kCellsPerThread];
#pragma unroll
  for (int w = 0; w < 6; ++w) {
    const int r = warp * kCellsPerThread + w;
    d[w] = s_in[0][r][lane];
    e[w] = s_in[1][r][lane];
    v[w] = s_in[2][r][lane];  // tangential in the y-sweep
    u[w] = s_in[3][r][lane];  // normal
  }
  float* mine = &s_out[0][warp * kCellsPerThread][lane];
#pragma unroll
  for (int r = 0; r < kCellsPerThread; ++r) {
    hm[r] = vm[r] = 0.f;
    if (!active) {
      mine[r * 32] = 0.f;
      mine[kYTileCells + r * 32] = 0.f;
      mine[2 * kYTileCells + r * 32] = 0.f;
    }
  }
  sweep_cells<1, true, false, false, true, false, FLAT, true>(sA, L, i0, active, 0, d, e, u, v, hm, vm, s_list,
                                                              &s_n, mine);
  __syncthreads();
  const unsigned cnt = s_n;
  bool bad = false;
  for (unsigned q = tid; q < cnt; q += blockDim.x) bad |= !general_to_tile<false>(sA, s_list[q], &s_out[0][0][0], r0, c0);
  if (bad) atomicOr(sA.status, ST_NAN);
  fence_proxy_async_smem();
  __syncthreads();
  if (tid == 0) {
    tma_store_2d(&M->srf_o, &s_out[0][0][0], c0, r0);
    tma_store_2d(&M->xu_o, &s_out[1][0][0], c0, r0);
    tma_store_2d(&M->yv_o, &s_out[2][0][0], c0, r0);
    bulk_commit();
    bulk_wait_read();
  }
}

}  // namespace cliffs
