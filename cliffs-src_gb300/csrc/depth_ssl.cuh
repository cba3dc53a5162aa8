// depth_ssl.cuh -- the bathymetry ratio limiter of the depth_ssl tool
// (depth_ssl/depth_ssl.f:222-362, setSSLim) on the device.
//
// A passage runs along every column, then along every row.  Each line is a
// sequential scan, because a node's rule reads its left neighbour's new
// value.  So a thread owns a line and streams it through a three-node window
// held in registers: the node ahead is read before the node behind is
// written back, in place.  Lines are independent, so the column pass has a
// thread per column (neighbouring threads read neighbouring addresses) and
// the row pass a thread per row.  The arithmetic is FP64 with IEEE sqrt and
// division, as in the reference, so results are bit-identical to a CPU run.
//   PHASE 0, open water: a node whose sqrt(depth) differs from a
//     neighbour's by more than the ratio alpha, with all three nodes at
//     least depmin deep, takes the mean of its neighbours' sqrt(depth).
//   PHASE 1, coastlines: a wet node with land on exactly one side is made
//     at least (its wet neighbour's depth) / alpha^2 deep.
#pragma once

namespace cliffs {

template <int PHASE, int DIR>
__global__ void k_depth_ssl(int nx, int ny, double* __restrict__ b, double alpha, double alp2, double depmin,
                            unsigned* count) {
  const int L = blockIdx.x * blockDim.x + threadIdx.x;
  const int lines = DIR == 0 ? nx : ny, len = DIR == 0 ? ny : nx;
  if (L >= lines || len < 3) return;
  const size_t st = DIR == 0 ? (size_t)nx : 1;
  double* line = DIR == 0 ? b + L : b + (size_t)L * nx;
  auto q_of = [&](double v, bool land) { return (PHASE == 0 && !land) ? sqrt(v) : v; };
  double v0 = line[0], v1 = line[st];
  bool l0 = v0 < depmin, l1 = v1 < depmin;
  double q0 = q_of(v0, l0), q1 = q_of(v1, l1);
  unsigned nodes = 0;
  for (int j = 1; j < len - 1; ++j) {
    const double v2 = line[(size_t)(j + 1) * st];
    const bool l2 = v2 < depmin;
    const double q2 = q_of(v2, l2);
    double out = v1;  // the node as it was, unless a rule moves it
    if (PHASE == 0) {
      if (!(l0 || l1 || l2)) {
        const double c1 = q2 / q1, c2 = q0 / q1;
        if (c1 > alpha || c2 > alpha) {
          q1 = (q0 + q2) / 2;
          out = q1 * q1;
          ++nodes;
        }
      }
    } else if (!l1 && (l2 != l0)) {
      const double dep = l2 ? q0 : q2;
      if (dep / q1 > alp2) {
        q1 = dep / alp2;
        out = q1;
        ++nodes;
      }
    }
    line[(size_t)j * st] = out;
    q0 = q1;
    l0 = l1;
    q1 = q2;
    l1 = l2;
    v1 = v2;
  }
  if (nodes) atomicAdd(count, nodes);
}

}  // namespace cliffs
