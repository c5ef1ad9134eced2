// step_kernels.cuh -- the kernels that are not templated on a system:
// ghost fill, dt and the step bookkeeping.  Included by runtime.cu only.
#pragma once

#include "batch.cuh"

namespace pypde {

__device__ __forceinline__ void k_boundaries_body(VBlock vb_, const double *__restrict__ u,
                             double *__restrict__ ub, const Geom &g, int N, int V,
                             const DevState *st) {
  if (!step_active(st))
    return;
  long long total = g.Cb * V;
  for (long long e = vb_.b * (long long)blockDim.x + threadIdx.x;
       e < total; e += (long long)vb_.n * blockDim.x) {
    long long idx = e / V;
    int v = (int)(e - idx * V);
    long long rem = idx, src = 0, mul = 1;
    for (int d = g.ndim - 1; d >= 0; d--) {
      int i = (int)(rem % g.nXb[d]);
      rem /= g.nXb[d];
      src += mul * renorm_index(i, N, g.bt[d], g.nX[d]);
      mul *= g.nX[d];
    }
    ub[e] = u[src * V + v];
  }
}

__global__ void k_boundaries(const double *__restrict__ u,
                             double *__restrict__ ub, const __grid_constant__ Geom g, int N, int V,
                             const DevState *st) {
  k_boundaries_body(VBlock{(long long)blockIdx.x, (long long)gridDim.x}, u, ub, g, N, V, st);
}

// dt from the reduced maximum (stepper.cpp:67-75)
__device__ __forceinline__ void dt_dev(DevState *st) {
  if (!step_active(st))
    return;
  double dt = st->cfl / st->max_speed;
  if (st->count <= 5)
    dt *= 0.2;
  if (st->t + dt > st->tf)
    dt = st->tf - st->t;
  st->dt = dt;
}
__global__ void k_dt(DevState *st) { dt_dev(st); }

// ---------------------------------------------------------------------
// Step bookkeeping (iterator.cpp:99-148).
// ---------------------------------------------------------------------
__device__ __forceinline__ void step_begin_dev(DevState *st) {
  st->active = (st->t < st->tf) &&
               (st->max_steps < 0 || st->count < st->max_steps) &&
               !st->nan_found;
  st->max_speed = 0.0;
  st->snap_slot = -1;
  st->nan_now = 0;
}
__global__ void k_step_begin(DevState *st) { step_begin_dev(st); }

// t += dt, count += 1, and the snapshot decision of iterator.cpp:136-139.
// Snapshots go to a ring of device slots the host drains between graph
// launches: slot = push % ring.
__device__ __forceinline__ void step_end_dev(DevState *st, int ring) {
  if (!step_active(st))
    return;
  st->t += st->dt;
  st->count += 1;
  if (st->push < st->ndt &&
      st->t >= double(st->push + 1) / double(st->ndt) * st->tf) {
    st->snap_slot = st->push % ring;
    st->push += 1;
  }
  if (st->nan_now)
    st->nan_found = 1;
}
__global__ void k_step_end(DevState *st, int ring) { step_end_dev(st, ring); }

// Batched bookkeeping: one thread per problem.
__global__ void kb_step_begin(const BatchProblem *P, int np) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < np)
    step_begin_dev(P[p].st);
}
__global__ void kb_dt(const BatchProblem *P, int np) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < np)
    dt_dev(P[p].st);
}
__global__ void kb_step_end(const BatchProblem *P, int np) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < np)
    step_end_dev(P[p].st, 1);
}

// Batched ghost fill (256 threads per tile).
__global__ void __launch_bounds__(256)
    kb_boundaries(const BatchProblem *P, TileQueue q, int per_pop) {
  drain(q, per_pop, [&](int p, VBlock vb) {
    const BatchProblem &b = P[p];
    k_boundaries_body(vb, b.u, b.ub, b.g, b.N, b.V, b.st);
  });
}

// Keep the state of the previous step (the NaN rows of iterator.cpp:141-145).
__global__ void k_copy_prev(const double *__restrict__ u,
                            double *__restrict__ uprev, long long n,
                            const DevState *st) {
  if (!step_active(st))
    return;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    uprev[i] = u[i];
}

// Copy u into its snapshot slot when k_step_end chose one.
__global__ void k_snapshot(const double *__restrict__ u,
                           double *__restrict__ ring, long long n,
                           const DevState *st) {
  if (!step_active(st) || st->snap_slot < 0)
    return;
  double *dst = ring + (long long)st->snap_slot * n;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    dst[i] = u[i];
}

// Training pairs for the warm start: after the predictor of step `count`
// (< nslots), copy per_slot sampled reconstruction cells' w and converged
// qh, and dt.  Sample j of slot s is cell (off_s + j stride) mod Cw.
__global__ void k_harvest(const double *__restrict__ w,
                          const double *__restrict__ qh, long long Cw, int nw,
                          int nq, const DevState *st, double *hw, double *hq,
                          double *hdt, long long stride, int nslots,
                          long long per_slot) {
  if (!step_active(st))
    return;
  const long long slot = st->count;
  if (slot >= nslots)
    return;
  const long long off = (slot * 7919 + 13) % stride;
  if (blockIdx.x == 0 && threadIdx.x == 0)
    hdt[slot] = st->dt;
  const long long tot = per_slot * (nw + nq);
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < tot;
       e += (long long)gridDim.x * blockDim.x) {
    const long long j = e / (nw + nq);
    const int k = (int)(e - j * (nw + nq));
    const long long cell = (off + j * stride) % Cw;
    if (k < nw)
      hw[(slot * per_slot + j) * nw + k] = w[cell * nw + k];
    else
      hq[(slot * per_slot + j) * nq + (k - nw)] = qh[cell * nq + (k - nw)];
  }
}

} // namespace pypde
