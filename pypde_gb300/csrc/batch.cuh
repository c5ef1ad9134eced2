// batch.cuh -- many independent problems in one launch per stage.
//
// Problems of one order N (possibly of different sizes, boundary types and
// end times) are stepped together: each stage is one persistent launch
// whose CTAs drain a work queue of tiles, tile = one block of the stage's
// one-problem launch (a VBlock of that problem), problems listed largest
// first so that the queue hands out the long work first.  A CTA pops
// `per_pop` consecutive tiles at a time; per_pop = 0 launches one hardware
// block per tile instead of the queue (the autotuner picks per stage).  The per-tile work is the one-problem kernels' bodies, unchanged,
// so a batched step gives the same bits as the same problem stepped alone.
// Not in the reference (one grid per pde_solver call).
#pragma once

#include "kernels.cuh"

namespace pypde {

// One problem of a batched step: its geometry and device buffers.
struct BatchProblem {
  Geom g;
  FaceIndex fi;
  int N, V;
  double *u, *ub, *w, *qh, *contrib, *cen, *wprod;
  // records of the two-launch Rusanov faces (kb_faces_pre, kb_faces_eig):
  // REC doubles per face point, component-major with the problem's face
  // points as stride; null where the faces run as one launch
  double *rec;
  // WENO pass d reads win[d] and writes wout[d] (the last writes w)
  const double *win[3];
  double *wout[3];
  long long wn1[3], wn3[3];
  int wmd[3], wn4[3];
  DevState *st;
};

// Tiles of one stage: problem p owns tiles [off[p], off[p+1]); head is a
// counter zeroed before the launch.
struct TileQueue {
  const long long *off;
  int np;
  unsigned long long *head;
};

// The problem owning tile t (binary search over the tile offsets).
__device__ __forceinline__ int tile_problem(const TileQueue &q, long long t) {
  int lo = 0, hi = q.np;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (q.off[mid] <= t)
      lo = mid;
    else
      hi = mid;
  }
  return lo;
}

// Pop per_pop tiles at a time until the queue is empty; body(p, vb) runs
// one tile of problem p with the whole CTA.  per_pop = 0: no queue, one
// hardware block per tile (the grid is the tile count).
template <class Body>
__device__ __forceinline__ void drain(const TileQueue &q, int per_pop,
                                      Body body) {
  if (per_pop == 0) {
    const long long t = blockIdx.x;
    if (t < q.off[q.np]) {
      const int p = tile_problem(q, t);
      body(p, VBlock{t - q.off[p], q.off[p + 1] - q.off[p]});
    }
    return;
  }
  __shared__ long long s_tile;
  const long long total = q.off[q.np];
  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0)
      s_tile = (long long)atomicAdd(q.head, (unsigned long long)per_pop);
    __syncthreads();
    const long long t0 = s_tile;
    if (t0 >= total)
      break;
    for (long long t = t0; t < t0 + per_pop && t < total; t++) {
      const int p = tile_problem(q, t);
      body(p, VBlock{t - q.off[p], q.off[p + 1] - q.off[p]});
      __syncthreads();
    }
  }
}

template <int N>
__global__ void __launch_bounds__(128)
    kb_weno(const BatchProblem *P, TileQueue q, int per_pop, int d, const __grid_constant__ Tables T) {
  drain(q, per_pop, [&](int p, VBlock vb) {
    const BatchProblem &b = P[p];
    k_weno_pass_body<N>(vb, b.win[d], b.wout[d], b.wn1[d], b.wmd[d], b.wn3[d],
                        b.wn4[d], b.V, T, b.st);
  });
}

template <class Sys, int N>
__global__ void __launch_bounds__(128)
    kb_cfl(const BatchProblem *P, TileQueue q, int per_pop, const __grid_constant__ Tables T) {
  drain(q, per_pop, [&](int p, VBlock vb) {
    const BatchProblem &b = P[p];
    k_cfl_body<Sys, N>(vb, b.w, b.g, T, b.wprod, b.st);
  });
}

template <class Sys, int N>
__global__ void kb_predictor(const BatchProblem *P, TileQueue q, int per_pop,
                             const __grid_constant__ Tables T) {
  drain(q, per_pop, [&](int p, VBlock vb) {
    const BatchProblem &b = P[p];
    k_predictor_body<Sys, N>(vb, b.w, b.qh, b.g, T, b.wprod, b.st);
  });
}

// flags: bit 0, start from the guess already in qh (the learned warm
// start of this order group); bit 1, FP32 sweeps first (mixed precision)
template <class Sys, int N>
__global__ void kb_newton(const BatchProblem *P, TileQueue q, int per_pop,
                          const __grid_constant__ Tables T, double tol,
                          int flags) {
  drain(q, per_pop, [&](int p, VBlock vb) {
    const BatchProblem &b = P[p];
    k_newton_body<Sys, N>(vb, b.w, b.qh, b.g, T, b.wprod, b.st, tol, flags & 1,
                          (flags >> 1) & 1);
  });
}

template <class Sys, int N, int FLUX>
__global__ void __launch_bounds__(128)
    kb_faces(const BatchProblem *P, TileQueue q, int per_pop, const __grid_constant__ Tables T) {
  drain(q, per_pop, [&](int p, VBlock vb) {
    const BatchProblem &b = P[p];
    k_faces_body<Sys, N, FLUX>(vb, b.qh, b.contrib, b.g, T, b.fi, b.st);
  });
}

// The Rusanov faces of a first-order flux system without B in two batched
// launches, as the one-problem step runs them (k_faces_pre, k_faces_eig):
// tile = 128 face points of one problem.
template <class Sys, int N>
__global__ void __launch_bounds__(128)
    kb_faces_pre(const BatchProblem *P, TileQueue q, int per_pop,
                 const __grid_constant__ Tables T) {
  drain(q, per_pop, [&](int p, VBlock vb) {
    const BatchProblem &b = P[p];
    if (!step_active(b.st))
      return;
    const long long n = b.fi.off[Sys::NDIM];
    const long long pt = vb.b * 128 + threadIdx.x;
    if (pt < n)
      face_pre_point<Sys, N>(pt, b.qh, b.rec + pt, n, b.g, T, b.fi, b.st->dt);
  });
}

template <class Sys, int N>
__global__ void __launch_bounds__(128, 4)
    kb_faces_eig(const BatchProblem *P, TileQueue q, int per_pop) {
  drain(q, per_pop, [&](int p, VBlock vb) {
    const BatchProblem &b = P[p];
    if (!step_active(b.st))
      return;
    const long long n = b.fi.off[Sys::NDIM];
    const long long pt = vb.b * 128 + threadIdx.x;
    if (pt < n)
      face_eig_point<Sys, N>(pt, b.rec + pt, n, b.contrib, b.fi);
  });
}

template <class Sys, int N>
__global__ void __launch_bounds__(128)
    kb_centers(const BatchProblem *P, TileQueue q, int per_pop, const __grid_constant__ Tables T) {
  drain(q, per_pop, [&](int p, VBlock vb) {
    const BatchProblem &b = P[p];
    k_centers_body<Sys, N>(vb, b.qh, b.cen, b.g, T, b.st);
  });
}

template <class Sys, int N>
__global__ void __launch_bounds__(256)
    kb_gather(const BatchProblem *P, TileQueue q, int per_pop, int use_centers,
              int use_faces) {
  drain(q, per_pop, [&](int p, VBlock vb) {
    const BatchProblem &b = P[p];
    k_gather_body<Sys, N>(vb, b.u, b.cen, b.contrib, b.g, b.fi, use_centers,
                          use_faces, b.st);
  });
}

} // namespace pypde
