// mlp.cuh -- the learned warm start of the stiff predictor.
//
// A per-cell MLP maps the WENO coefficients of a cell and log10(dt/tau) to
// the correction qh - w of the space-time predictor at every space-time
// node; qh = w + correction is the initial guess of the Newton iteration
// (k_newton with guess = 1), which still iterates to the same residual
// tolerance and falls back to the plain guess when the residual does not
// fall.  Not in the reference (its predictor always starts from w,
// dg.cpp:187-199).
//
// Network: x (K1) -> SiLU(W1 x + b1) (128) -> SiLU(W2 . + b2) (128)
//          -> W3 . + b3 (NO).  Weights in BF16, every GEMM operand rounded
// to BF16 (round to nearest even), FP32 accumulation on the tensor cores
// (mma.sync m16n8k16), bias and activation in FP32.
//
// Features of a cell, in this order (computed in FP64, then FP32):
//   mean_v   = (sum_idx w[idx][v]) * (1/Nd)             v < V
//   dev      = w[idx][v] - mean_v                       idx < Nd, v < V
//   lg       = log10(dt) - mean_{tau_var}  (log10(dt) when tau_var < 0)
//   lr       = log10(r), r below
// normalised as x = (f - x_mean) * x_scale (FP32); then the deviations are
// made homogeneous: r = max(sqrt(sum of their squares / (Nd V)), 1e-30)
// and each is divided by r (times 1/r), so the network sees the shape of
// the cell's data and its magnitude only through lr.  Padded with zeros to
// K1.  Output o = (t Nd + idx) V + v: correction = (y_o * y_scale_o +
// y_mean_o) * r -- the predictor's correction scales with the cell's
// variation, and so does the network's error.
#pragma once

#include "batch.cuh"
#include "kernels.cuh"

namespace pypde {

constexpr int MLP_H = 128; // hidden width
constexpr int MLP_PAD = 8; // row padding of the weights in shared memory

template <class Sys, int N> struct MlpShape {
  static constexpr int V = Sys::V, D = Sys::NDIM;
  static constexpr int Nd = IPow<N, D>::value, NT = N * Nd;
  static constexpr int FEAT = V + Nd * V + 2;
  static constexpr int K1 = (FEAT + 15) / 16 * 16;
  static constexpr int NO = (NT * V + 7) / 8 * 8;
  static constexpr bool OK = K1 <= 128 && NO <= 256;
  static constexpr int WARPS = 8, CELLS = WARPS * 16; // one m16 tile per warp
  static constexpr int S1 = K1 + MLP_PAD, S2 = MLP_H + MLP_PAD;
  static constexpr int W_ELEMS = MLP_H * S1 + MLP_H * S2 + NO * S2; // bf16
  static constexpr int P_FLOATS = 2 * MLP_H + NO + 2 * K1 + 2 * NO;
  static constexpr size_t SMEM = (size_t)((W_ELEMS + 1) / 2) * 4 +
                                 (size_t)(P_FLOATS + CELLS * K1 + CELLS) * 4;
};

// Device copy of a trained network (pointers into one allocation).
struct MlpModel {
  const unsigned short *W1, *W2, *W3; // bf16 bits, [H][k1], [H][H], [no][H]
  const float *b1, *b2, *b3;          // [H], [H], [no]
  const float *x_mean, *x_scale;      // [k1]
  const float *y_mean, *y_scale;      // [no]
  int k1, no, tau_var;
};

// FP32 -> BF16, round to nearest even (NaN kept a quiet NaN).
__device__ __forceinline__ unsigned short f32_to_bf16(float f) {
  unsigned int u = __float_as_uint(f);
  if ((u & 0x7fffffffu) > 0x7f800000u)
    return (unsigned short)((u >> 16) | 0x40u);
  u += 0x7fffu + ((u >> 16) & 1u);
  return (unsigned short)(u >> 16);
}

__device__ __forceinline__ unsigned int pack_bf16(float lo, float hi) {
  return (unsigned int)f32_to_bf16(lo) | ((unsigned int)f32_to_bf16(hi) << 16);
}

__device__ __forceinline__ float silu(float z) {
  return z / (1.0f + expf(-z));
}

// D = A B + D, A 16x16 (row), B 16x8 (col), BF16 in, FP32 accumulate.
// Fragments (g = lane / 4, c = lane % 4): a0 (g, 2c..2c+1), a1 (g+8, 2c..),
// a2 (g, 2c+8..), a3 (g+8, 2c+8..); b0 (k 2c..2c+1, n g), b1 (k 2c+8.., n g);
// d0,d1 (g, 2c..2c+1), d2,d3 (g+8, 2c..2c+1).
__device__ __forceinline__ void mma_bf16_16816(float d[4], const unsigned int a[4],
                                               unsigned int b0, unsigned int b1) {
  asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
               "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
               : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
               : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// One hidden layer on a warp's 16 rows: acc (16 n-tiles of 8) = A (KT
// k-tiles) x W^T with W [128][stride] in shared memory; then bias, SiLU and
// repacking of the FP32 accumulators into the A fragments of the next
// layer (8 k-tiles over the 128 hidden units).
template <int KT>
__device__ __forceinline__ void mlp_hidden(const unsigned int (&a)[KT][4],
                                           const unsigned short *W, int stride,
                                           const float *bias, int lane,
                                           unsigned int (&out)[8][4]) {
  const int g = lane >> 2, c = lane & 3;
#pragma unroll
  for (int j = 0; j < 8; j++) {
    float acc[2][4];
#pragma unroll
    for (int h = 0; h < 2; h++) {
      const int nt = 2 * j + h;
#pragma unroll
      for (int i = 0; i < 4; i++)
        acc[h][i] = 0.0f;
      const unsigned short *wr = W + (nt * 8 + g) * stride + 2 * c;
#pragma unroll
      for (int kt = 0; kt < KT; kt++) {
        unsigned int b0 = *(const unsigned int *)(wr + kt * 16);
        unsigned int b1 = *(const unsigned int *)(wr + kt * 16 + 8);
        mma_bf16_16816(acc[h], a[kt], b0, b1);
      }
    }
    const int n0 = 16 * j + 2 * c, n1 = n0 + 8;
    out[j][0] = pack_bf16(silu(acc[0][0] + bias[n0]), silu(acc[0][1] + bias[n0 + 1]));
    out[j][1] = pack_bf16(silu(acc[0][2] + bias[n0]), silu(acc[0][3] + bias[n0 + 1]));
    out[j][2] = pack_bf16(silu(acc[1][0] + bias[n1]), silu(acc[1][1] + bias[n1 + 1]));
    out[j][3] = pack_bf16(silu(acc[1][2] + bias[n1]), silu(acc[1][3] + bias[n1 + 1]));
  }
}

// Shared-memory layout of the guess: the network (staged once per block)
// and each warp's 16 cells of features and scales.
struct MlpSmem {
  unsigned short *W1, *W2, *W3;
  float *b1, *b2, *b3, *xm, *xs, *ym, *ys, *F, *R;
};

// Stage the network in shared memory (all threads; ends with a barrier).
template <class Sys, int N>
__device__ __forceinline__ MlpSmem mlp_stage(const MlpModel &m) {
  using S = MlpShape<Sys, N>;
  constexpr int K1 = S::K1, NO = S::NO;
  extern __shared__ float4 mlp_smem4[];
  MlpSmem sm;
  sm.W1 = (unsigned short *)mlp_smem4;
  sm.W2 = sm.W1 + MLP_H * S::S1;
  sm.W3 = sm.W2 + MLP_H * S::S2;
  float *sp = (float *)mlp_smem4 + (S::W_ELEMS + 1) / 2;
  sm.b1 = sp;
  sm.b2 = sm.b1 + MLP_H;
  sm.b3 = sm.b2 + MLP_H;
  sm.xm = sm.b3 + NO;
  sm.xs = sm.xm + K1;
  sm.ym = sm.xs + K1;
  sm.ys = sm.ym + NO;
  sm.F = sm.ys + NO;              // [CELLS][K1]
  sm.R = sm.F + S::CELLS * K1;    // [CELLS] per-cell scale r
  for (int i = threadIdx.x; i < MLP_H * K1; i += blockDim.x)
    sm.W1[(i / K1) * S::S1 + i % K1] = m.W1[i];
  for (int i = threadIdx.x; i < MLP_H * MLP_H; i += blockDim.x)
    sm.W2[(i / MLP_H) * S::S2 + i % MLP_H] = m.W2[i];
  for (int i = threadIdx.x; i < NO * MLP_H; i += blockDim.x)
    sm.W3[(i / MLP_H) * S::S2 + i % MLP_H] = m.W3[i];
  for (int i = threadIdx.x; i < MLP_H; i += blockDim.x) {
    sm.b1[i] = m.b1[i];
    sm.b2[i] = m.b2[i];
  }
  for (int i = threadIdx.x; i < NO; i += blockDim.x) {
    sm.b3[i] = m.b3[i];
    sm.ym[i] = m.y_mean[i];
    sm.ys[i] = m.y_scale[i];
  }
  for (int i = threadIdx.x; i < K1; i += blockDim.x) {
    sm.xm[i] = m.x_mean[i];
    sm.xs[i] = m.x_scale[i];
  }
  __syncthreads();
  return sm;
}

// One tile of CELLS reconstruction cells (cells tile*CELLS ...) of one
// grid, each warp 16 of them: qh = w + the network's correction at every
// space-time node.  lg_dt = log10 of the step's dt.
template <class Sys, int N>
__device__ __forceinline__ void mlp_guess_tile(const MlpSmem &sm,
                                               const double *__restrict__ w,
                                               double *__restrict__ qh,
                                               long long Cw, int tau_var,
                                               double lg_dt, long long tile) {
  using S = MlpShape<Sys, N>;
  constexpr int V = S::V, Nd = S::Nd, NT = S::NT, K1 = S::K1, NO = S::NO;
  constexpr int KT1 = K1 / 16;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int gr = lane >> 2, c = lane & 3;
  float *F = sm.F + warp * 16 * K1;
  float *R = sm.R + warp * 16;
  const long long cell0 = tile * S::CELLS + warp * 16;
  if (lane < 16) {
    const long long cell = cell0 + lane;
    float *f = F + lane * K1;
    if (cell < Cw) {
      const double *wc = w + cell * Nd * V;
      double tau_mean = 0.0;
      for (int v = 0; v < V; v++) {
        double s = wc[v];
        for (int idx = 1; idx < Nd; idx++)
          s += wc[idx * V + v];
        const double mean = s * (1.0 / Nd);
        f[v] = (float)mean;
        for (int idx = 0; idx < Nd; idx++)
          f[V + idx * V + v] = (float)(wc[idx * V + v] - mean);
        if (v == tau_var)
          tau_mean = mean;
      }
      f[V + Nd * V] = (float)(tau_var >= 0 ? lg_dt - tau_mean : lg_dt);
      for (int k = 0; k < S::FEAT - 1; k++)
        f[k] = (f[k] - sm.xm[k]) * sm.xs[k];
      float ss = 0.0f;
      for (int k = V; k < V + Nd * V; k++)
        ss += f[k] * f[k];
      const float r = fmaxf(sqrtf(ss * (1.0f / (float)(Nd * V))), 1e-30f);
      const float rr = 1.0f / r;
      for (int k = V; k < V + Nd * V; k++)
        f[k] = f[k] * rr;
      f[S::FEAT - 1] = (log10f(r) - sm.xm[S::FEAT - 1]) * sm.xs[S::FEAT - 1];
      for (int k = S::FEAT; k < K1; k++)
        f[k] = 0.0f;
      R[lane] = r;
    } else {
      for (int k = 0; k < K1; k++)
        f[k] = 0.0f;
      R[lane] = 0.0f;
    }
  }
  __syncwarp();
  unsigned int a1[KT1][4];
#pragma unroll
  for (int kt = 0; kt < KT1; kt++) {
    const float *r0 = F + gr * K1 + kt * 16 + 2 * c;
    const float *r1 = r0 + 8 * K1;
    a1[kt][0] = pack_bf16(r0[0], r0[1]);
    a1[kt][1] = pack_bf16(r1[0], r1[1]);
    a1[kt][2] = pack_bf16(r0[8], r0[9]);
    a1[kt][3] = pack_bf16(r1[8], r1[9]);
  }
  __syncwarp();
  unsigned int a2[8][4], a3[8][4];
  mlp_hidden<KT1>(a1, sm.W1, S::S1, sm.b1, lane, a2);
  mlp_hidden<8>(a2, sm.W2, S::S2, sm.b2, lane, a3);
  // output layer, one n-tile of 8 outputs at a time
#pragma unroll 1
  for (int nt = 0; nt < NO / 8; nt++) {
    float acc[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    const unsigned short *wr = sm.W3 + (nt * 8 + gr) * S::S2 + 2 * c;
#pragma unroll
    for (int kt = 0; kt < 8; kt++) {
      unsigned int b0 = *(const unsigned int *)(wr + kt * 16);
      unsigned int b1 = *(const unsigned int *)(wr + kt * 16 + 8);
      mma_bf16_16816(acc, a3[kt], b0, b1);
    }
#pragma unroll
    for (int h = 0; h < 2; h++) {
      const long long cell = cell0 + gr + 8 * h;
      if (cell >= Cw)
        continue;
      const float r = R[gr + 8 * h];
#pragma unroll
      for (int e = 0; e < 2; e++) {
        const int o = nt * 8 + 2 * c + e;
        if (o >= NT * V)
          continue;
        const float y = acc[2 * h + e] + sm.b3[o];
        const float corr = (y * sm.ys[o] + sm.ym[o]) * r;
        const int idx = (o / V) % Nd, v = o % V;
        qh[cell * NT * V + o] = w[(cell * Nd + idx) * V + v] + (double)corr;
      }
    }
  }
  __syncwarp(); // R and F are rewritten by the next tile
}

// The guess kernel: a persistent grid over tiles of 128 reconstruction
// cells, one warp per 16 cells; the weights are staged in shared memory
// once per block.  Writes qh = w + correction for every space-time node.
template <class Sys, int N>
__global__ void __launch_bounds__(256)
    k_mlp_guess(const double *__restrict__ w, double *__restrict__ qh, Geom g,
                MlpModel m, const DevState *st) {
  using S = MlpShape<Sys, N>;
  if (!step_active(st))
    return;
  const MlpSmem sm = mlp_stage<Sys, N>(m);
  const double lg_dt = log10(st->dt);
  for (long long tile = blockIdx.x; tile * S::CELLS < g.Cw; tile += gridDim.x)
    mlp_guess_tile<Sys, N>(sm, w, qh, g.Cw, m.tau_var, lg_dt, tile);
}

// The learned warm start of an order group: the network is staged in
// shared memory once per CTA, then every tile (128 reconstruction cells of
// one problem) writes qh = w + the network's correction, as k_mlp_guess
// does for that problem alone.
template <class Sys, int N>
__global__ void __launch_bounds__(256)
    kb_mlp_guess(const BatchProblem *P, TileQueue q, int per_pop, MlpModel m) {
  const MlpSmem sm = mlp_stage<Sys, N>(m);
  drain(q, per_pop, [&](int p, VBlock vb) {
    const BatchProblem &b = P[p];
    if (step_active(b.st))
      mlp_guess_tile<Sys, N>(sm, b.w, b.qh, b.g.Cw, m.tau_var, log10(b.st->dt),
                             vb.b);
  });
}

} // namespace pypde
