// Strips of one step (host only).
//
// The predictor of a step (k_newton or k_predictor) runs over the w-cells
// in S strips of whole blocks, cell order being row-major over the
// reconstruction grid nXw (axis 0 slowest).  Once strips 0..s are done, the
// faces whose two cells lie in them are known, and k_faces runs on them on
// a second stream while strip s+1 is predicted.  The two kernels leave
// each other's registers and shared memory free (k_newton is bounded by
// its shared memory, k_faces by its registers), so an SM holds blocks of
// both and the FP64 pipe idles less than with one kernel after the other.
//
// A face of direction d is numbered by its low-side w-cell O (fv.cpp:
// 124-198 walks the same faces): O_d in [0, n_d], O_e in [1, n_e] for
// e != d, row-major over that box with axis 0 slowest.  Its first index i0
// is O_0 for d = 0 and O_0 - 1 otherwise, and its cells lie in w-rows
// i0 and i0 + 1 (d = 0) or in w-row i0 + 1 (d != 0).  So a face is ready
// once w-rows 0..i0+1 are complete, whatever its direction, and the faces
// ready after a strip are a range of i0 in every direction: a contiguous
// range of face points.
#pragma once

namespace pypde {

constexpr int MAX_STRIPS = 32;

struct StripPlan {
  int S = 1;
  // predictor strip s: blocks [blk[s], blk[s+1])
  long long blk[MAX_STRIPS + 1] = {};
  // face points released by strip s: n[s][d] points of direction d from
  // lo[s][d] on
  long long lo[MAX_STRIPS][3] = {}, n[MAX_STRIPS][3] = {};
};

// S strips over Cw cells in blocks of cpb cells (fewer when the grid has
// fewer blocks).  nX: interior cells per axis, nXw = nX + 2, off[d]: first
// face point of direction d, N: order (N time nodes, N^(ndim-1) transverse
// nodes per face).
inline void plan_strips(int S, int ndim, const int *nX, const int *nXw,
                        long long Cw, int cpb, int N, const long long *off,
                        StripPlan *p) {
  const long long blocks = (Cw + cpb - 1) / cpb;
  if (S > MAX_STRIPS)
    S = MAX_STRIPS;
  if (S > blocks)
    S = (int)blocks;
  if (S < 1)
    S = 1;
  p->S = S;
  for (int s = 0; s <= S; s++)
    p->blk[s] = blocks * s / S;
  long long row = 1; // cells per w-row
  for (int e = 1; e < ndim; e++)
    row *= nXw[e];
  long long nodes = N; // face points per face: N time x N^(ndim-1) nodes
  for (int e = 1; e < ndim; e++)
    nodes *= N;
  long long per[3] = {0, 0, 0}, cnt[3] = {0, 0, 0};
  for (int d = 0; d < ndim; d++) {
    long long f = 1; // faces per value of i0
    for (int e = 1; e < ndim; e++)
      f *= (e == d) ? nX[e] + 1 : nX[e];
    per[d] = f * nodes;
    cnt[d] = (d == 0) ? nX[0] + 1 : nX[0];
  }
  long long prev[3] = {0, 0, 0};
  for (int s = 0; s < S; s++) {
    long long done = p->blk[s + 1] * cpb;
    if (done > Cw || s == S - 1)
      done = Cw;
    const long long rows = done / row; // complete w-rows
    for (int d = 0; d < 3; d++) {
      long long hi = rows - 1;
      if (hi < 0)
        hi = 0;
      if (hi > cnt[d])
        hi = cnt[d];
      if (d >= ndim)
        hi = 0;
      p->lo[s][d] = (d < ndim ? off[d] : 0) + prev[d] * per[d];
      p->n[s][d] = (hi - prev[d]) * per[d];
      prev[d] = hi;
    }
  }
}

} // namespace pypde
