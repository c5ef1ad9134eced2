// mlp_train.cu -- training kernels of the warm-start network and the device
// copy of a trained network.
//
// The GEMM rounds both operands to BF16 (round to nearest even) as it stages
// them in shared memory and accumulates in FP32 on the tensor cores with
// the same mma.sync m16n8k16 instruction and the same k order as the fused
// inference kernel (k_mlp_guess), so the training forward pass and the
// in-solver inference compute the same numbers.
#include "mlp.cuh"
#include "runtime.h"

#include <cstring>
#include <vector>

namespace pypde {

constexpr int GB_M = 64, GB_N = 64, GB_K = 32, GB_S = GB_K + 8;

// C[M][N] = sum_k A(m,k) B(k,n) with A(m,k) = A[m sam + k sak] and
// B(k,n) = B[k sbk + n sbn].  Block (bx, by, bz): the 64x64 tile (by, bx)
// over k in [bz kchunk, (bz+1) kchunk).  With part non-null the raw sums go
// to part[bz][M][N]; otherwise C = sum + bias and act = SiLU(C) (each
// optional).
__global__ void __launch_bounds__(128)
    k_gemm_bf16(const float *__restrict__ A, long long sam, long long sak,
                const float *__restrict__ B, long long sbk, long long sbn,
                float *__restrict__ C, int M, int N, int K, int kchunk,
                const float *__restrict__ bias, float *__restrict__ act,
                float *__restrict__ part) {
  __shared__ unsigned short sA[GB_M * GB_S], sB[GB_N * GB_S];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int g = lane >> 2, c = lane & 3;
  const int wm = warp >> 1, wn = warp & 1;
  const long long m0 = (long long)blockIdx.y * GB_M;
  const long long n0 = (long long)blockIdx.x * GB_N;
  const int k0 = blockIdx.z * kchunk;
  const int k1 = min(K, k0 + kchunk);
  float acc[2][4][4];
#pragma unroll
  for (int i = 0; i < 2; i++)
#pragma unroll
    for (int j = 0; j < 4; j++)
#pragma unroll
      for (int e = 0; e < 4; e++)
        acc[i][j][e] = 0.0f;
  for (int kb = k0; kb < k1; kb += GB_K) {
    for (int e = tid; e < GB_M * GB_K; e += 128) {
      int r, kk;
      if (sak == 1) {
        r = e / GB_K;
        kk = e % GB_K;
      } else {
        kk = e / GB_M;
        r = e % GB_M;
      }
      const long long m = m0 + r;
      const int k = kb + kk;
      const float v = (m < M && k < k1) ? A[m * sam + (long long)k * sak] : 0.0f;
      sA[r * GB_S + kk] = f32_to_bf16(v);
    }
    for (int e = tid; e < GB_N * GB_K; e += 128) {
      int cc, kk;
      if (sbn == 1) {
        kk = e / GB_N;
        cc = e % GB_N;
      } else {
        cc = e / GB_K;
        kk = e % GB_K;
      }
      const long long n = n0 + cc;
      const int k = kb + kk;
      const float v = (n < N && k < k1) ? B[(long long)k * sbk + n * sbn] : 0.0f;
      sB[cc * GB_S + kk] = f32_to_bf16(v);
    }
    __syncthreads();
#pragma unroll
    for (int ks = 0; ks < GB_K / 16; ks++) {
      unsigned int a[2][4];
#pragma unroll
      for (int mt = 0; mt < 2; mt++) {
        const unsigned short *r0 = sA + (wm * 32 + mt * 16 + g) * GB_S + ks * 16 + 2 * c;
        const unsigned short *r1 = r0 + 8 * GB_S;
        a[mt][0] = *(const unsigned int *)r0;
        a[mt][1] = *(const unsigned int *)r1;
        a[mt][2] = *(const unsigned int *)(r0 + 8);
        a[mt][3] = *(const unsigned int *)(r1 + 8);
      }
#pragma unroll
      for (int nt = 0; nt < 4; nt++) {
        const unsigned short *br = sB + (wn * 32 + nt * 8 + g) * GB_S + ks * 16 + 2 * c;
        const unsigned int b0 = *(const unsigned int *)br;
        const unsigned int b1 = *(const unsigned int *)(br + 8);
#pragma unroll
        for (int mt = 0; mt < 2; mt++)
          mma_bf16_16816(acc[mt][nt], a[mt], b0, b1);
      }
    }
    __syncthreads();
  }
#pragma unroll
  for (int mt = 0; mt < 2; mt++)
#pragma unroll
    for (int nt = 0; nt < 4; nt++)
#pragma unroll
      for (int e = 0; e < 4; e++) {
        const long long m = m0 + wm * 32 + mt * 16 + g + (e >= 2 ? 8 : 0);
        const long long n = n0 + wn * 32 + nt * 8 + 2 * c + (e & 1);
        if (m >= M || n >= N)
          continue;
        if (part) {
          part[((long long)blockIdx.z * M + m) * N + n] = acc[mt][nt][e];
        } else {
          const float z = acc[mt][nt][e] + (bias ? bias[n] : 0.0f);
          if (C)
            C[m * N + n] = z;
          if (act)
            act[m * N + n] = silu(z);
        }
      }
}

// Sum of the split-K partial tiles in split order, then bias and SiLU.
__global__ void k_splitk_epilogue(const float *__restrict__ part, int splits,
                                  int M, int N, const float *__restrict__ bias,
                                  float *__restrict__ C, float *__restrict__ act) {
  const long long total = (long long)M * N;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    float s = part[i];
    for (int z = 1; z < splits; z++)
      s += part[(long long)z * total + i];
    const float v = s + (bias ? bias[i % N] : 0.0f);
    if (C)
      C[i] = v;
    if (act)
      act[i] = silu(v);
  }
}

// dZ = dA * SiLU'(Z), SiLU'(z) = s (1 + z (1 - s)) with s = 1 / (1 + e^-z).
__global__ void k_silu_grad(const float *__restrict__ dA,
                            const float *__restrict__ Z, float *__restrict__ dZ,
                            long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const float z = Z[i];
    const float s = 1.0f / (1.0f + expf(-z));
    dZ[i] = dA[i] * (s * (1.0f + z * (1.0f - s)));
  }
}

// out[n] = sum_m X[m][n], a fixed-order tree per column (deterministic).
__global__ void k_colsum(const float *__restrict__ X, int M, int N,
                         float *__restrict__ out) {
  __shared__ float red[256];
  const int n = blockIdx.x;
  float s = 0.0f;
  for (int m = threadIdx.x; m < M; m += blockDim.x)
    s += X[(long long)m * N + n];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int h = blockDim.x / 2; h > 0; h >>= 1) {
    if (threadIdx.x < h)
      red[threadIdx.x] += red[threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x == 0)
    out[n] = red[0];
}

// Host FP32 -> BF16, the same rounding as f32_to_bf16.
static unsigned short host_bf16(float f) {
  unsigned int u;
  std::memcpy(&u, &f, 4);
  if ((u & 0x7fffffffu) > 0x7f800000u)
    return (unsigned short)((u >> 16) | 0x40u);
  u += 0x7fffu + ((u >> 16) & 1u);
  return (unsigned short)(u >> 16);
}

static int cuda_fail(cudaError_t e, const char *what) {
  set_error(std::string(what) + ": " + cudaGetErrorString(e));
  return -2;
}

int mlp_gemm(const float *A, long long sam, long long sak, const float *B,
             long long sbk, long long sbn, float *C, int M, int N, int K,
             int splits, float *work, const float *bias, float *act,
             cudaStream_t s) {
  if (M <= 0 || N <= 0 || K <= 0 || splits < 1 || (splits > 1 && !work)) {
    set_error("mlp_gemm: bad sizes or missing split-K workspace");
    return -1;
  }
  int kchunk = (K + splits - 1) / splits;
  kchunk = (kchunk + GB_K - 1) / GB_K * GB_K;
  splits = (K + kchunk - 1) / kchunk;
  dim3 grid((N + GB_N - 1) / GB_N, (M + GB_M - 1) / GB_M, splits);
  if (grid.y > 65535u) {
    set_error("mlp_gemm: M too large");
    return -1;
  }
  k_gemm_bf16<<<grid, 128, 0, s>>>(A, sam, sak, B, sbk, sbn, C, M, N, K,
                                   kchunk, bias, act,
                                   splits > 1 ? work : nullptr);
  if (splits > 1) {
    long long tot = (long long)M * N;
    unsigned blocks = (unsigned)std::min<long long>((tot + 255) / 256, 152 * 8);
    k_splitk_epilogue<<<blocks, 256, 0, s>>>(work, splits, M, N, bias, C, act);
  }
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? 0 : cuda_fail(e, "mlp_gemm");
}

int mlp_silu_grad(const float *dA, const float *Z, float *dZ, long long n,
                  cudaStream_t s) {
  if (n <= 0)
    return 0;
  unsigned blocks = (unsigned)std::min<long long>((n + 255) / 256, 152 * 16);
  k_silu_grad<<<blocks, 256, 0, s>>>(dA, Z, dZ, n);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? 0 : cuda_fail(e, "mlp_silu_grad");
}

int mlp_colsum(const float *X, int M, int N, float *out, cudaStream_t s) {
  if (M <= 0 || N <= 0) {
    set_error("mlp_colsum: bad sizes");
    return -1;
  }
  k_colsum<<<N, 256, 0, s>>>(X, M, N, out);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? 0 : cuda_fail(e, "mlp_colsum");
}

// ----------------------------------------------------------------------
// Device copy of a trained network.
// ----------------------------------------------------------------------
int warm_start_create(const WarmStartDesc &d, WarmStart **out) {
  const int H = MLP_H, k1 = d.k1, no = d.no;
  if (k1 <= 0 || no <= 0 || k1 % 16 || no % 8) {
    set_error("warm start: k1 must be a multiple of 16 and no of 8");
    return -1;
  }
  std::vector<unsigned short> wb((size_t)H * k1 + (size_t)H * H + (size_t)no * H);
  size_t o = 0;
  for (size_t i = 0; i < (size_t)H * k1; i++)
    wb[o++] = host_bf16(d.W1[i]);
  for (size_t i = 0; i < (size_t)H * H; i++)
    wb[o++] = host_bf16(d.W2[i]);
  for (size_t i = 0; i < (size_t)no * H; i++)
    wb[o++] = host_bf16(d.W3[i]);
  std::vector<float> pf;
  pf.insert(pf.end(), d.b1, d.b1 + H);
  pf.insert(pf.end(), d.b2, d.b2 + H);
  pf.insert(pf.end(), d.b3, d.b3 + no);
  pf.insert(pf.end(), d.x_mean, d.x_mean + k1);
  pf.insert(pf.end(), d.x_scale, d.x_scale + k1);
  pf.insert(pf.end(), d.y_mean, d.y_mean + no);
  pf.insert(pf.end(), d.y_scale, d.y_scale + no);
  size_t wbytes = (wb.size() * 2 + 255) / 256 * 256;
  size_t bytes = wbytes + pf.size() * 4;
  cudaError_t e = cudaSetDevice(d.device);
  if (e != cudaSuccess)
    return cuda_fail(e, "warm start: cudaSetDevice");
  void *mem = nullptr;
  e = cudaMalloc(&mem, bytes);
  if (e != cudaSuccess)
    return cuda_fail(e, "warm start: cudaMalloc");
  e = cudaMemcpy(mem, wb.data(), wb.size() * 2, cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy((char *)mem + wbytes, pf.data(), pf.size() * 4,
                   cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    cudaFree(mem);
    return cuda_fail(e, "warm start: upload");
  }
  WarmStart *ws = new WarmStart();
  ws->device = d.device;
  ws->mem = mem;
  const unsigned short *wp = (const unsigned short *)mem;
  const float *fp = (const float *)((char *)mem + wbytes);
  MlpModel &m = ws->model;
  m.W1 = wp;
  m.W2 = wp + (size_t)H * k1;
  m.W3 = m.W2 + (size_t)H * H;
  m.b1 = fp;
  m.b2 = fp + H;
  m.b3 = fp + 2 * H;
  m.x_mean = m.b3 + no;
  m.x_scale = m.x_mean + k1;
  m.y_mean = m.x_scale + k1;
  m.y_scale = m.y_mean + no;
  m.k1 = k1;
  m.no = no;
  m.tau_var = d.tau_var;
  *out = ws;
  return 0;
}

void warm_start_free(WarmStart *ws) {
  if (!ws)
    return;
  int prev = 0;
  cudaGetDevice(&prev);
  cudaSetDevice(ws->device);
  cudaFree(ws->mem);
  cudaSetDevice(prev);
  delete ws;
}

} // namespace pypde
