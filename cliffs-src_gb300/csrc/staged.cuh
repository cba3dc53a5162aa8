// staged.cuh -- persistent sweep kernels whose window loads arrive in shared
// memory through the bulk-copy (TMA) engine, one tile ahead of the compute.
//
// fast_kernel (sweep.cuh) issues its loads and then waits for them: with 6
// blocks of 4 warps per SM (80 registers a thread) the wait is the largest
// stall of both sweeps.  Here each block stays resident and walks tiles
// blockIdx.x, blockIdx.x + gridDim.x, ...; while it computes tile i, the copy
// engine fills the other of two shared-memory stages with tile i+1.  Thread 0
// issues the copies; every thread waits on the stage's mbarrier (bounded by
// StageCtl::wait_ns) and reads its window from shared memory.  The compute,
// the stores and the block-local general path are sweep_cells, shared with
// fast_kernel, so the two kernels give identical results.
//
//   staged_x  x-sweep tiles of 512 cells of a row (4 per thread).  Per field
//             one 1-D bulk copy of the row segment plus a 16-byte chunk on
//             each side, which holds the neighbour cells.  Tiles are numbered
//             segment-major (all rows' first segments, then the second ...),
//             so a block's tiles cover every segment: the coast of a basin
//             that runs across the rows falls in one segment of each row, and
//             with row-major numbering a grid whose size is a multiple of the
//             segment count would give all of those tiles to the same blocks.
//   staged_y  y-sweep tiles of 32 columns x 16 rows (a warp per 4 rows, a lane
//             per column).  Per field one 2-D tensor-map copy of 32 x 18 rows,
//             the tile plus one halo row each side; rows outside the grid read
//             0.  The max-wave fields come as 32 x 16 boxes.
//
// Measured on GB300 these kernels are the slower choice, and fast_kernel stays
// the default.  The loads' wait does go (long-scoreboard stalls fall from 2.2
// to 0.9 per issue).  But the loop's state pushes the 80-register budget of 6
// blocks per SM into spills, or, at 96 registers, down to 5 blocks.  The
// per-tile barrier also costs what the hardware's block scheduler gave for
// free.  On the 4320 x 2160 spherical grid the x-sweep takes 105 us against
// 93 us and the y-sweep 94.5 against 94.
#pragma once
#include "sweep.cuh"
#include "tma.cuh"

namespace cliffs {

constexpr int kStagedThreads = 128;
constexpr int kXTile = kStagedThreads * kCellsPerThread;  // cells of a row per x tile
constexpr int kXRow = kXTile + 8;                           // + one 16-byte chunk each side
constexpr int kYRows = (kStagedThreads / 32) * kCellsPerThread;  // rows per y tile
constexpr int kYWin = kYRows + 2;                                // + one halo row each side

enum : unsigned { ST_STALL = 2u };  // a stage wait ran out

struct StageCtl {
  unsigned long long wait_ns;  // limit of one stage wait
  unsigned extra;              // bytes a stage waits for beyond its copies: 0,
                               // except in the timeout self-test
};

// Tensor maps of the y-sweep's fields (row-major, nx x ny, row pitch of the
// grid): window fields with a 32 x kYWin box, max-wave fields 32 x kYRows.
struct YMaps {
  CUtensorMap dep, srf, xu, yv;
  CUtensorMap hmax, velmax;
};

// Waits for the stage of tile i (the block's i-th tile); on a timeout every
// thread of the block learns of it, thread 0 records it and waits (bounded)
// for the copies of the other stage if they were issued, and the caller
// leaves the kernel.  The barrier also orders the block: every thread is done
// with tile i-1 (its compute, its reads of the other stage) when it returns.
__device__ __forceinline__ bool stage_wait(uint64_t* bar, int i, bool next_issued, const SweepArgs& A,
                                           const StageCtl& S) {
  const bool ok = mbar_wait_ns(&bar[i & 1], (uint32_t)(i >> 1) & 1u, S.wait_ns);
  if (__syncthreads_or(!ok)) {
    if (threadIdx.x == 0) {
      atomicOr(A.status, ST_STALL);
      if (next_issued) mbar_wait_ns(&bar[(i + 1) & 1], (uint32_t)((i + 1) >> 1) & 1u, S.wait_ns);
    }
    return false;
  }
  return true;
}

// The block's list of cells that need the full rules, per tile: tile i
// appends to list[i & 1] and count[i % 3]; its cells are finished by the whole
// block after the next tile's barrier (which also orders them after the tile's
// fast stores), while the next tile appends to the other list.  The count of
// tile i+1 is zeroed after tile i's barrier: its last reader, the tail of
// tile i-2, ran before it.
struct BlockList {
  uint32_t list[2][kXTile];
  unsigned count[3];
};

template <int DIR>
__device__ __forceinline__ void block_list_tail(const SweepArgs& A, const BlockList& B, int i) {
  const unsigned cnt = B.count[i % 3];
  for (unsigned k = threadIdx.x; k < cnt; k += blockDim.x) general_store<DIR, false>(A, B.list[i & 1][k]);
}

__global__ void __launch_bounds__(kStagedThreads, 6) staged_x(const SweepArgs A, const StageCtl S) {
  __shared__ __align__(128) float sx[2][4][kXRow];  // [stage][dep, srf, xu, yv][cell + 4 - c0]
  __shared__ BlockList B;
  __shared__ __align__(8) uint64_t bar[2];
  const int n = A.n;
  const int segs = (n + kXTile - 1) / kXTile;
  const int T = segs * A.nlines;
  const int tid = threadIdx.x, lane = tid & 31;
  if (tid == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    B.count[0] = B.count[1] = B.count[2] = 0u;
    fence_mbar_init();
  }
  __syncthreads();
  // copies of tile t into stage s: columns [c0 - 4, c0 + 516) of row L, cut
  // to the row (its pitch); every bound is a multiple of 4 cells (16 bytes)
  auto issue = [&](int t, int s) {
    const int L = t % A.nlines + 1, seg = t / A.nlines;
    const int c0 = seg * kXTile;
    const int lo = seg > 0 ? c0 - 4 : c0;
    const int hi = min(c0 + kXTile + 4, A.pitch);
    const uint32_t bytes = (uint32_t)(hi - lo) * 4u;
    const size_t at = (size_t)(L - 1) * (size_t)A.pitch + (size_t)lo;
    const int off = lo - (c0 - 4);
    mbar_expect_tx(&bar[s], 4u * bytes + S.extra);
    bulk_load(&sx[s][0][off], A.dep + at, bytes, &bar[s]);
    bulk_load(&sx[s][1][off], A.srf + at, bytes, &bar[s]);
    bulk_load(&sx[s][2][off], A.xu + at, bytes, &bar[s]);
    bulk_load(&sx[s][3][off], A.yv + at, bytes, &bar[s]);
  };
  int t = blockIdx.x, i = 0;
  if (tid == 0 && t < T) issue(t, 0);
  for (; t < T; ++i, t += gridDim.x) {
    const int s = i & 1;
    const bool next = t + (int)gridDim.x < T;
    if (!stage_wait(bar, i, false, A, S)) return;
    if (tid == 0) {
      B.count[(i + 1) % 3] = 0u;
      if (next) issue(t + gridDim.x, s ^ 1);  // the stage of tile i-1, free since the barrier
    }
    if (i > 0) block_list_tail<0>(A, B, i - 1);
    const int L = t % A.nlines + 1;
    const int c0 = (t / A.nlines) * kXTile;
    const int i0 = c0 + tid * kCellsPerThread + 1;
    const bool active = i0 <= n;
    const size_t q0 = (size_t)(L - 1) * (size_t)A.pitch + (size_t)(i0 - 1);
    const int b = 4 + tid * kCellsPerThread;  // the thread's cells at b..b+3
    float d[6], e[6], u[6], v[6];
    float hm[kCellsPerThread], vm[kCellsPerThread];
    const float4 D4 = *reinterpret_cast<const float4*>(&sx[s][0][b]);
    const float4 E4 = *reinterpret_cast<const float4*>(&sx[s][1][b]);
    const float4 X4 = *reinterpret_cast<const float4*>(&sx[s][2][b]);
    const float4 Y4 = *reinterpret_cast<const float4*>(&sx[s][3][b]);
    d[1] = D4.x; d[2] = D4.y; d[3] = D4.z; d[4] = D4.w;
    e[1] = E4.x; e[2] = E4.y; e[3] = E4.z; e[4] = E4.w;
    u[1] = X4.x; u[2] = X4.y; u[3] = X4.z; u[4] = X4.w;
    v[1] = Y4.x; v[2] = Y4.y; v[3] = Y4.z; v[4] = Y4.w;
    // neighbours from the adjacent lanes; the warp's end lanes read them from
    // the stage, clamped to the line
    d[0] = __shfl_up_sync(0xffffffffu, D4.w, 1);
    e[0] = __shfl_up_sync(0xffffffffu, E4.w, 1);
    u[0] = __shfl_up_sync(0xffffffffu, X4.w, 1);
    v[0] = __shfl_up_sync(0xffffffffu, Y4.w, 1);
    d[5] = __shfl_down_sync(0xffffffffu, D4.x, 1);
    e[5] = __shfl_down_sync(0xffffffffu, E4.x, 1);
    u[5] = __shfl_down_sync(0xffffffffu, X4.x, 1);
    v[5] = __shfl_down_sync(0xffffffffu, Y4.x, 1);
    if (lane == 0) {
      const int bl = i0 > 1 ? b - 1 : b;
      d[0] = sx[s][0][bl]; e[0] = sx[s][1][bl]; u[0] = sx[s][2][bl]; v[0] = sx[s][3][bl];
    }
    if (lane == 31 || i0 + 4 > n) {  // past the line's end the stage may hold no copy
      const int br = active ? b + (min(i0 + 4, n) - i0) : b;
      d[5] = sx[s][0][br]; e[5] = sx[s][1][br]; u[5] = sx[s][2][br]; v[5] = sx[s][3][br];
    }
    float4 H4 = make_float4(0.f, 0.f, 0.f, 0.f), V4 = H4;
    if (A.hmax && active) {  // fused only when no y-sweep follows (1-D runs)
      H4 = ld_state4<false>(A.hmax + q0);
      V4 = ld_state4<false>(A.velmax + q0);
    }
    hm[0] = H4.x; hm[1] = H4.y; hm[2] = H4.z; hm[3] = H4.w;
    vm[0] = V4.x; vm[1] = V4.y; vm[2] = V4.z; vm[3] = V4.w;
    sweep_cells<0, true, false, false>(A, L, i0, active, q0, d, e, u, v, hm, vm, B.list[s], &B.count[i % 3]);
  }
  __syncthreads();
  if (i > 0) block_list_tail<0>(A, B, i - 1);
}

__global__ void __launch_bounds__(kStagedThreads, 6)
    staged_y(const SweepArgs A, const __grid_constant__ YMaps M, const StageCtl S) {
  __shared__ __align__(128) float sy[2][4][kYWin][32];   // [stage][dep, srf, xu, yv][row + 1 - r0][col - x0]
  __shared__ __align__(128) float sm[2][2][kYRows][32];  // [stage][hmax, velmax][row - r0][col - x0]
  __shared__ BlockList B;
  __shared__ __align__(8) uint64_t bar[2];
  const int n = A.n;  // rows
  const int RG = (n + kYRows - 1) / kYRows;
  const int T = RG * ((A.nlines + 31) / 32);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const bool fmax = A.hmax != nullptr;
  if (tid == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    B.count[0] = B.count[1] = B.count[2] = 0u;
    fence_mbar_init();
  }
  __syncthreads();
  constexpr uint32_t kWinBytes = kYWin * 32 * 4, kMaxBytes = kYRows * 32 * 4;
  auto issue = [&](int t, int s) {
    const int x = (t / RG) * 32, y = (t % RG) * kYRows;
    mbar_expect_tx(&bar[s], 4u * kWinBytes + (fmax ? 2u * kMaxBytes : 0u) + S.extra);
    tma_load_2d(&sy[s][0][0][0], &M.dep, &bar[s], x, y - 1);
    tma_load_2d(&sy[s][1][0][0], &M.srf, &bar[s], x, y - 1);
    tma_load_2d(&sy[s][2][0][0], &M.xu, &bar[s], x, y - 1);
    tma_load_2d(&sy[s][3][0][0], &M.yv, &bar[s], x, y - 1);
    if (fmax) {
      tma_load_2d(&sm[s][0][0][0], &M.hmax, &bar[s], x, y);
      tma_load_2d(&sm[s][1][0][0], &M.velmax, &bar[s], x, y);
    }
  };
  int t = blockIdx.x, i = 0;
  if (tid == 0 && t < T) issue(t, 0);
  for (; t < T; ++i, t += gridDim.x) {
    const int s = i & 1;
    const bool next = t + (int)gridDim.x < T;
    if (!stage_wait(bar, i, false, A, S)) return;
    if (tid == 0) {
      B.count[(i + 1) % 3] = 0u;
      if (next) issue(t + gridDim.x, s ^ 1);
    }
    if (i > 0) block_list_tail<1>(A, B, i - 1);
    const int L = (t / RG) * 32 + lane + 1;
    const int i0 = (t % RG) * kYRows + warp * kCellsPerThread + 1;
    const bool active = L <= A.nlines && i0 <= n;
    float d[6], e[6], u[6], v[6];
    float hm[kCellsPerThread], vm[kCellsPerThread];
#pragma unroll
    for (int w = 0; w < 6; ++w) {
      const int r = warp * kCellsPerThread + w;
      d[w] = sy[s][0][r][lane];
      e[w] = sy[s][1][r][lane];
      v[w] = sy[s][2][r][lane];  // tangential in the y-sweep
      u[w] = sy[s][3][r][lane];  // normal
    }
#pragma unroll
    for (int r = 0; r < kCellsPerThread; ++r) {
      hm[r] = fmax ? sm[s][0][warp * kCellsPerThread + r][lane] : 0.f;
      vm[r] = fmax ? sm[s][1][warp * kCellsPerThread + r][lane] : 0.f;
    }
    sweep_cells<1, true, false, false>(A, L, i0, active, 0, d, e, u, v, hm, vm, B.list[s], &B.count[i % 3]);
  }
  __syncthreads();
  if (i > 0) block_list_tail<1>(A, B, i - 1);
}

}  // namespace cliffs
