// batch.cuh -- many grids (scenarios) stepped together.
//
// An ensemble of independent runs (one source scenario per grid, grids of
// uneven size) has the same work per step as one run of the ensemble's total
// size, but each grid alone fills only part of the GPU and pays two launches
// per step.  Here every scenario's sweep is cut into the same tiles the
// single-grid kernels use (sweep_tile: 128 threads, 512 cells of a row in the
// x-sweep, 32 columns x 16 rows in the y-sweep), the tiles of all scenarios
// form one flat list per sweep direction, and a block maps a list index to its
// scenario by bisection over the per-scenario tile offsets.  Two schedules:
//   batch_persistent  one cooperative launch for many steps; the blocks loop
//                     over the x tiles, meet at a grid barrier, loop over the
//                     y tiles, meet again, and so on;
//   batch_phase<DIR>  one launch per sweep direction and step covering every
//                     scenario, for capture in a CUDA graph.
// A scenario's tiles do the same arithmetic as its own sweep launches, so a
// batched run is bit-identical to stepping the grids one by one.  Two
// argument sets: "fused" (the y-sweep updates the max-wave fields with its
// outputs), for a scenario's first step from a fresh state and for steps of
// a rising source, and "fold" (the x-sweep folds the previous step's end
// state in, the y-sweep has no max-wave code), for every other step.
#pragma once
#include "sweep.cuh"

namespace cliffs {

struct YTileMaps;

struct BatchArgs {
  const SweepArgs* args;  // [2k] x-sweep, [2k+1] y-sweep of scenario k
  const int* off;         // [dir * (n+1) + k]: first tile of scenario k; [n] the total
  const int* gx;          // [dir * n + k]: tiles along the first grid dimension
  int n;                  // scenarios
  int steps;              // steps of one persistent launch
  unsigned* bar;          // grid barrier counter, zero at launch
  unsigned* err;          // set when a barrier wait runs out
  unsigned long long wait_ns;  // limit of one barrier wait
  unsigned extra;         // arrivals a barrier waits for beyond the grid's
                          // blocks: 0, except in the timeout self-test
  int span[2];            // tile shape: single-grid tiles per list entry, along
                          // the rows (x-sweep: rows of 512 cells; y-sweep:
                          // groups of 16 rows of 32 columns)
  const YTileMaps* ymaps;  // per scenario, the y-sweep's tensor maps (batch_tile_y)
};

constexpr int kBatchThreads = 128;
constexpr unsigned long long kBarrierNs = 2000000000ull;  // default limit, 2 s: far above any sweep phase

__device__ __forceinline__ int batch_scenario(const int* off, int n, int t) {
  int lo = 0, hi = n;  // off[lo] <= t < off[hi]
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (__ldg(off + mid) <= t)
      lo = mid;
    else
      hi = mid;
  }
  return lo;
}

// The list entries first, first + stride, ... of one sweep direction over
// all scenarios.  An entry is B.span[DIR] single-grid tiles along the rows: x,
// span consecutive rows of one 512-cell column chunk; y, span consecutive
// 16-row groups of one 32-column group.  The scenario's arguments are staged
// in shared memory once per entry.  MULTI = false: entries of one tile
// (span 1), with no loop around the tile's code, which keeps the loop's
// state out of the tile's register budget.
// FLAT: every scenario's lines of this direction have uniform spacing and no
// metric term (the single-grid kernels' flat variant: the same bits).
template <int DIR, bool COH, bool MAXOUT, bool MULTI = true, bool FLAT = false>
__device__ __forceinline__ void batch_tiles(const BatchArgs& B, int first, int stride) {
  __shared__ SweepArgs sA;
  const int* off = B.off + DIR * (B.n + 1);
  const int total = __ldg(off + B.n);
  const int span = B.span[DIR];
  for (int t = first; t < total; t += stride) {
    const int k = batch_scenario(off, B.n, t);
    const int local = t - __ldg(off + k);
    const int g = __ldg(B.gx + DIR * B.n + k);
    __syncthreads();  // the previous tile is done with sA and its shared list
    if (threadIdx.x == 0) sA = B.args[2 * k + DIR];
    __syncthreads();
    if (!MULTI) {
      sweep_tile<DIR, true, COH, true, MAXOUT, FLAT>(sA, local % g, local / g);
    } else if (DIR == 0) {  // g: column chunks; rows (local / g) * span ...
      const int bx = local % g, by0 = (local / g) * span;
      for (int r = 0; r < span && by0 + r < sA.nlines; ++r) sweep_tile<0, true, COH, true, MAXOUT>(sA, bx, by0 + r);
    } else {  // g: entries along the column, each span row groups of 16
      const int bx0 = (local % g) * span, by = local / g;
      const int groups = (sA.n + (kBatchThreads / 32) * kCellsPerThread - 1) / ((kBatchThreads / 32) * kCellsPerThread);
      for (int r = 0; r < span && bx0 + r < groups; ++r) sweep_tile<1, true, COH, true, MAXOUT>(sA, bx0 + r, by);
    }
  }
}

__device__ __forceinline__ unsigned ld_acquire_gpu(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Grid-wide barrier of a cooperative launch (every block is resident).  Each
// block's thread 0 publishes the block's writes (fence, then arrival count)
// and waits until all blocks of this epoch arrived (plus `extra`), for at most
// wait_ns; after that, or when another block already gave up, it sets *err and
// the block leaves the kernel (returns false).
__device__ __forceinline__ bool grid_sync(unsigned* bar, unsigned nblocks, unsigned& epoch, unsigned* err,
                                          unsigned long long wait_ns, unsigned extra) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    atomicAdd(bar, 1u);
    const unsigned target = (epoch + 1u) * nblocks + extra;
    const unsigned long long t0 = global_ns();
    int ok = 1;
    while (ld_acquire_gpu(bar) < target) {
      if (ld_acquire_gpu(err) != 0u) {
        ok = 0;
        break;
      }
      if (global_ns() - t0 > wait_ns) {
        atomicOr(err, 1u);
        ok = 0;
        break;
      }
      __nanosleep(64);
    }
    __threadfence();
    s_ok = ok;
  }
  __syncthreads();
  ++epoch;
  return s_ok != 0;
}

// MAXOUT = false: the y-sweeps carry no max-wave update (the argument set
// whose x-sweeps fold the previous step's end state in, hmax_in).
template <bool MAXOUT>
__global__ void __launch_bounds__(kBatchThreads, 6) batch_persistent(const BatchArgs B) {
  unsigned epoch = 0;
  for (int s = 0; s < B.steps; ++s) {
    batch_tiles<0, true, false>(B, blockIdx.x, gridDim.x);
    if (!grid_sync(B.bar, gridDim.x, epoch, B.err, B.wait_ns, B.extra)) return;
    batch_tiles<1, true, MAXOUT>(B, blockIdx.x, gridDim.x);
    if (!grid_sync(B.bar, gridDim.x, epoch, B.err, B.wait_ns, B.extra)) return;
  }
}

// 64 registers, 8 blocks per SM: with the max-wave fold this measured 3 %
// faster than 80 registers and 6 blocks (2.34 against 2.41 ms per step on the
// 256-scenario ensemble), spills included.  MULTI: entries of more than one
// tile (B.span[DIR] > 1); the one-tile variant has no loop around the tile
// (2.34 against 2.70 ms per step with the loop at span 1).
template <int DIR, bool MAXOUT, bool MULTI, bool FLAT = false>
__global__ void __launch_bounds__(kBatchThreads, 8) batch_phase(const BatchArgs B) {
  batch_tiles<DIR, false, MAXOUT, MULTI, FLAT>(B, blockIdx.x, gridDim.x);
}

}  // namespace cliffs
