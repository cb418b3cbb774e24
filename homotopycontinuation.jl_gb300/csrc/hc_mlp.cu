// hc_mlp.cu — the step-proposal network: a 12→64→64→2 MLP with BF16 operands and FP32
// accumulation on the tensor cores (mma.sync m16n8k16), trained on the GPU by these kernels.
//
// Parameters (FP32 master copy, HC_MLP_NPARAMS floats, row-major):
//   W1[64][12] b1[64] W2[64][64] b2[64] W3[2][64] b3[2]
// Model: o = W3 relu(W2 relu(W1 x + b1) + b2) + b3, x the 12 normalised step features.
// Loss of a logged step (features x, tried log-multiplier ℓ, accepted y ∈ {0,1}):
//   k = softplus(o2) + 0.05, z = k (o1 − ℓ), p = σ(z), L = softplus(z) − y z   (BCE of p vs y)
// i.e. o1 is the log step multiplier at which acceptance turns over, k its sharpness.
// No counterpart in the reference: its step control is the closed-form rule this network
// proposes alternatives to (src/tracker.jl:541-588).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/hcgpu.h"

namespace {

constexpr int NI = 12, NH = 64, NO = 2;
constexpr int OFF_W1 = 0, OFF_B1 = OFF_W1 + NH * NI, OFF_W2 = OFF_B1 + NH, OFF_B2 = OFF_W2 + NH * NH,
              OFF_W3 = OFF_B2 + NH, OFF_B3 = OFF_W3 + NO * NH, NPARAMS = OFF_B3 + NO;
constexpr int WARPS = 4, ROWS_PER_WARP = 16;

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<uint32_t*>(&v);
}

// D = A(16x16 bf16, row) * B(16x8 bf16, col) + C (f32)
__device__ __forceinline__ void mma16816(float* d, const uint32_t* a, const uint32_t* b) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// Fragment helpers for m16n8k16 (g = lane/4, q = lane%4):
//   A: a0 (g, 2q..2q+1) a1 (g+8, 2q..) a2 (g, 2q+8..) a3 (g+8, 2q+8..)
//   B: b0 (k=2q..2q+1, n=g) b1 (k=2q+8.., n=g)
//   C: c0,c1 (g, 2q..2q+1) c2,c3 (g+8, 2q..2q+1)
// `A(r, k)` and `B(k, n)` are float accessors; out-of-range elements must return 0.
template <class FA>
__device__ __forceinline__ void load_a(uint32_t* a, FA A) {
  int lane = threadIdx.x & 31, g = lane >> 2, q = lane & 3;
  a[0] = pack_bf16(A(g, 2 * q), A(g, 2 * q + 1));
  a[1] = pack_bf16(A(g + 8, 2 * q), A(g + 8, 2 * q + 1));
  a[2] = pack_bf16(A(g, 2 * q + 8), A(g, 2 * q + 9));
  a[3] = pack_bf16(A(g + 8, 2 * q + 8), A(g + 8, 2 * q + 9));
}
template <class FB>
__device__ __forceinline__ void load_b(uint32_t* b, FB B) {
  int lane = threadIdx.x & 31, g = lane >> 2, q = lane & 3;
  b[0] = pack_bf16(B(2 * q, g), B(2 * q + 1, g));
  b[1] = pack_bf16(B(2 * q + 8, g), B(2 * q + 9, g));
}
template <class FC>
__device__ __forceinline__ void store_c(const float* c, FC C) {
  int lane = threadIdx.x & 31, g = lane >> 2, q = lane & 3;
  C(g, 2 * q, c[0]);
  C(g, 2 * q + 1, c[1]);
  C(g + 8, 2 * q, c[2]);
  C(g + 8, 2 * q + 1, c[3]);
}

__device__ __forceinline__ float softplus(float x) { return x > 20.f ? x : log1pf(expf(x)); }
__device__ __forceinline__ float sigmoid(float x) { return 1.f / (1.f + expf(-x)); }

struct WarpTile {
  float X[16][NI + 4];
  float H1[16][NH];
  float H2[16][NH];
  float dO[16][8];
  float dH2[16][NH];
  float dH1[16][NH];
};

// forward of 16 rows (rows beyond `nrows` are zero); fills T.H1, T.H2 and returns O in o[16][2]
__device__ void forward_tile(WarpTile& T, const float* P, float (*O)[2]) {
  const int lane = threadIdx.x & 31;
  // layer 1: H1 = relu(X W1ᵀ + b1); K = 12 padded to 16
  for (int nt = 0; nt < NH / 8; ++nt) {
    float c[4] = {0, 0, 0, 0};
    uint32_t a[4], b[2];
    load_a(a, [&](int r, int k) { return k < NI ? T.X[r][k] : 0.f; });
    load_b(b, [&](int k, int n) { return k < NI ? P[OFF_W1 + (nt * 8 + n) * NI + k] : 0.f; });
    mma16816(c, a, b);
    store_c(c, [&](int r, int n, float v) { T.H1[r][nt * 8 + n] = fmaxf(v + P[OFF_B1 + nt * 8 + n], 0.f); });
  }
  __syncwarp();
  // layer 2: H2 = relu(H1 W2ᵀ + b2); K = 64
  for (int nt = 0; nt < NH / 8; ++nt) {
    float c[4] = {0, 0, 0, 0};
    for (int kt = 0; kt < NH / 16; ++kt) {
      uint32_t a[4], b[2];
      load_a(a, [&](int r, int k) { return T.H1[r][kt * 16 + k]; });
      load_b(b, [&](int k, int n) { return P[OFF_W2 + (nt * 8 + n) * NH + kt * 16 + k]; });
      mma16816(c, a, b);
    }
    store_c(c, [&](int r, int n, float v) { T.H2[r][nt * 8 + n] = fmaxf(v + P[OFF_B2 + nt * 8 + n], 0.f); });
  }
  __syncwarp();
  // layer 3: O = H2 W3ᵀ + b3; N = 2 padded to 8
  float c[4] = {0, 0, 0, 0};
  for (int kt = 0; kt < NH / 16; ++kt) {
    uint32_t a[4], b[2];
    load_a(a, [&](int r, int k) { return T.H2[r][kt * 16 + k]; });
    load_b(b, [&](int k, int n) { return n < NO ? P[OFF_W3 + n * NH + kt * 16 + k] : 0.f; });
    mma16816(c, a, b);
  }
  store_c(c, [&](int r, int n, float v) {
    if (n < NO) O[r][n] = v + P[OFF_B3 + n];
  });
  __syncwarp();
  (void)lane;
}

// params: FP32 master weights (read as BF16 operands). One warp per 16 rows.
constexpr size_t FWD_SMEM = sizeof(WarpTile) * WARPS + sizeof(float) * WARPS * 16 * 2;
constexpr size_t GRAD_SMEM = FWD_SMEM + sizeof(float) * NPARAMS;

__global__ void __launch_bounds__(32 * WARPS) mlp_forward_kernel(const float* __restrict__ X, int B,
                                                                 const float* __restrict__ P, float* __restrict__ out) {
  extern __shared__ __align__(16) unsigned char dsm[];
  WarpTile* tiles = (WarpTile*)dsm;
  float(*Os)[16][2] = (float(*)[16][2])(dsm + sizeof(WarpTile) * WARPS);
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  WarpTile& T = tiles[w];
  for (int base = (blockIdx.x * WARPS + w) * 16; base < B; base += gridDim.x * WARPS * 16) {
    for (int e = lane; e < 16 * (NI + 4); e += 32) {
      int r = e / (NI + 4), k = e % (NI + 4);
      T.X[r][k] = (base + r < B && k < NI) ? X[(size_t)(base + r) * NI + k] : 0.f;
    }
    __syncwarp();
    forward_tile(T, P, Os[w]);
    for (int e = lane; e < 32; e += 32) {
      int r = e / 2, n = e % 2;
      if (base + r < B) out[(size_t)(base + r) * NO + n] = Os[w][r][n];
    }
    __syncwarp();
  }
}

// loss + gradients of a batch; gradient accumulated (FP32 atomics) into G[NPARAMS], loss sum
// into *loss. Weight gradients of a CTA are first summed in shared memory.
__global__ void __launch_bounds__(32 * WARPS) mlp_grad_kernel(const float* __restrict__ X, const float* __restrict__ L,
                                                              const float* __restrict__ Y, int B,
                                                              const float* __restrict__ P, float* __restrict__ G,
                                                              float* __restrict__ loss) {
  extern __shared__ __align__(16) unsigned char dsm[];
  WarpTile* tiles = (WarpTile*)dsm;
  float(*Os)[16][2] = (float(*)[16][2])(dsm + sizeof(WarpTile) * WARPS);
  float* gs = (float*)(dsm + FWD_SMEM);
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int i = threadIdx.x; i < NPARAMS; i += blockDim.x) gs[i] = 0.f;
  __syncthreads();
  WarpTile& T = tiles[w];
  const float invB = 1.f / (float)B;
  float lsum = 0.f;
  for (int base = (blockIdx.x * WARPS + w) * 16; base < B; base += gridDim.x * WARPS * 16) {
    for (int e = lane; e < 16 * (NI + 4); e += 32) {
      int r = e / (NI + 4), k = e % (NI + 4);
      T.X[r][k] = (base + r < B && k < NI) ? X[(size_t)(base + r) * NI + k] : 0.f;
    }
    __syncwarp();
    forward_tile(T, P, Os[w]);
    // dL/dO per row (mean over the batch)
    if (lane < 16) {
      int r = lane;
      float d1 = 0.f, d2 = 0.f;
      if (base + r < B) {
        float o1 = Os[w][r][0], o2 = Os[w][r][1];
        float ell = L[base + r], y = Y[base + r];
        float k = softplus(o2) + 0.05f;
        float z = k * (o1 - ell);
        float p = sigmoid(z);
        lsum += softplus(z) - y * z;
        float dz = (p - y) * invB;
        d1 = dz * k;
        d2 = dz * (o1 - ell) * sigmoid(o2);
      }
      T.dO[r][0] = d1;
      T.dO[r][1] = d2;
      for (int n = 2; n < 8; ++n) T.dO[r][n] = 0.f;
    }
    __syncwarp();
    // dW3, db3 (CUDA cores: 2×64 outputs, 16 rows)
    for (int e = lane; e < NO * NH; e += 32) {
      int j = e / NH, u = e % NH;
      float s = 0.f;
      for (int r = 0; r < 16; ++r) s += T.dO[r][j] * T.H2[r][u];
      atomicAdd(&gs[OFF_W3 + j * NH + u], s);
    }
    if (lane < NO) {
      float s = 0.f;
      for (int r = 0; r < 16; ++r) s += T.dO[r][lane];
      atomicAdd(&gs[OFF_B3 + lane], s);
    }
    // dH2 = dO W3 ⊙ [H2 > 0]
    for (int e = lane; e < 16 * NH; e += 32) {
      int r = e / NH, u = e % NH;
      float s = T.dO[r][0] * P[OFF_W3 + u] + T.dO[r][1] * P[OFF_W3 + NH + u];
      T.dH2[r][u] = T.H2[r][u] > 0.f ? s : 0.f;
    }
    __syncwarp();
    // db2
    for (int u = lane; u < NH; u += 32) {
      float s = 0.f;
      for (int r = 0; r < 16; ++r) s += T.dH2[r][u];
      atomicAdd(&gs[OFF_B2 + u], s);
    }
    // dW2 = dH2ᵀ H1 : M = 64 (u), N = 64 (v), K = 16 (rows)
    for (int mt = 0; mt < NH / 16; ++mt)
      for (int nt = 0; nt < NH / 8; ++nt) {
        float c[4] = {0, 0, 0, 0};
        uint32_t a[4], b[2];
        load_a(a, [&](int m, int k) { return T.dH2[k][mt * 16 + m]; });
        load_b(b, [&](int k, int n) { return T.H1[k][nt * 8 + n]; });
        mma16816(c, a, b);
        store_c(c, [&](int m, int n, float v) { atomicAdd(&gs[OFF_W2 + (mt * 16 + m) * NH + nt * 8 + n], v); });
      }
    // dH1 = dH2 W2 ⊙ [H1 > 0] : M = 16 rows, N = 64 (v), K = 64 (u)
    for (int nt = 0; nt < NH / 8; ++nt) {
      float c[4] = {0, 0, 0, 0};
      for (int kt = 0; kt < NH / 16; ++kt) {
        uint32_t a[4], b[2];
        load_a(a, [&](int r, int k) { return T.dH2[r][kt * 16 + k]; });
        load_b(b, [&](int k, int n) { return P[OFF_W2 + (kt * 16 + k) * NH + nt * 8 + n]; });
        mma16816(c, a, b);
      }
      store_c(c, [&](int r, int n, float v) { T.dH1[r][nt * 8 + n] = T.H1[r][nt * 8 + n] > 0.f ? v : 0.f; });
    }
    __syncwarp();
    // db1
    for (int u = lane; u < NH; u += 32) {
      float s = 0.f;
      for (int r = 0; r < 16; ++r) s += T.dH1[r][u];
      atomicAdd(&gs[OFF_B1 + u], s);
    }
    // dW1 = dH1ᵀ X : M = 64 (u), N = 12 → 16 (i), K = 16 (rows)
    for (int mt = 0; mt < NH / 16; ++mt)
      for (int nt = 0; nt < 2; ++nt) {
        float c[4] = {0, 0, 0, 0};
        uint32_t a[4], b[2];
        load_a(a, [&](int m, int k) { return T.dH1[k][mt * 16 + m]; });
        load_b(b, [&](int k, int n) { return (nt * 8 + n) < NI ? T.X[k][nt * 8 + n] : 0.f; });
        mma16816(c, a, b);
        store_c(c, [&](int m, int n, float v) {
          if (nt * 8 + n < NI) atomicAdd(&gs[OFF_W1 + (mt * 16 + m) * NI + nt * 8 + n], v);
        });
      }
    __syncwarp();
  }
  for (int o = 16; o; o >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
  if (lane == 0) atomicAdd(loss, lsum * invB);
  __syncthreads();
  for (int i = threadIdx.x; i < NPARAMS; i += blockDim.x) atomicAdd(&G[i], gs[i]);
}

__global__ void adam_kernel(float* P, float* M, float* V, const float* G, int n, float lr, float b1, float b2,
                            float eps, float bc1, float bc2, float wd) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float g = G[i] + wd * P[i];
  float m = b1 * M[i] + (1.f - b1) * g;
  float v = b2 * V[i] + (1.f - b2) * g * g;
  M[i] = m;
  V[i] = v;
  P[i] -= lr * (m / bc1) / (sqrtf(v / bc2) + eps);
}

}  // namespace

extern "C" {

// Number of FP32 parameters of the step-proposal network (layout in hc_mlp.cu).
int hc_mlp_num_params(void) { return NPARAMS; }

// out[B×2] = network(X[B×12]) with BF16 operands / FP32 accumulation; device pointers.
int hc_mlp_forward(const float* d_X, int B, const float* d_params, float* d_out, void* stream) {
  if (B < 0 || (B > 0 && (!d_X || !d_params || !d_out))) return HC_ERR_INVALID_ARG;
  if (B == 0) return HC_OK;
  int blocks = (B + WARPS * 16 - 1) / (WARPS * 16);
  if (blocks > 4096) blocks = 4096;
  if (cudaFuncSetAttribute(mlp_forward_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)FWD_SMEM) !=
      cudaSuccess)
    return HC_ERR_CUDA;
  mlp_forward_kernel<<<blocks, 32 * WARPS, FWD_SMEM, (cudaStream_t)stream>>>(d_X, B, d_params, d_out);
  return cudaGetLastError() == cudaSuccess ? HC_OK : HC_ERR_CUDA;
}

// Mean BCE loss and its gradient over a batch (device pointers; d_grad and d_loss are
// overwritten). X[B×12] features, L[B] tried log-multipliers, Y[B] accepted (0/1).
int hc_mlp_grad(const float* d_X, const float* d_L, const float* d_Y, int B, const float* d_params, float* d_grad,
                float* d_loss, void* stream) {
  if (B <= 0 || !d_X || !d_L || !d_Y || !d_params || !d_grad || !d_loss) return HC_ERR_INVALID_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  if (cudaMemsetAsync(d_grad, 0, NPARAMS * sizeof(float), s) != cudaSuccess) return HC_ERR_CUDA;
  if (cudaMemsetAsync(d_loss, 0, sizeof(float), s) != cudaSuccess) return HC_ERR_CUDA;
  int blocks = (B + WARPS * 16 - 1) / (WARPS * 16);
  if (blocks > 1024) blocks = 1024;
  if (cudaFuncSetAttribute(mlp_grad_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)GRAD_SMEM) !=
      cudaSuccess)
    return HC_ERR_CUDA;
  mlp_grad_kernel<<<blocks, 32 * WARPS, GRAD_SMEM, s>>>(d_X, d_L, d_Y, B, d_params, d_grad, d_loss);
  return cudaGetLastError() == cudaSuccess ? HC_OK : HC_ERR_CUDA;
}

// One Adam step (bias-corrected; L2 weight decay added to the gradient) on the FP32 master
// parameters.
int hc_mlp_adam(float* d_params, float* d_m, float* d_v, const float* d_grad, int step, float lr, float weight_decay,
                void* stream) {
  if (!d_params || !d_m || !d_v || !d_grad || step < 1) return HC_ERR_INVALID_ARG;
  const float b1 = 0.9f, b2 = 0.999f;
  float bc1 = 1.f - powf(b1, (float)step), bc2 = 1.f - powf(b2, (float)step);
  adam_kernel<<<(NPARAMS + 255) / 256, 256, 0, (cudaStream_t)stream>>>(d_params, d_m, d_v, d_grad, NPARAMS, lr, b1,
                                                                        b2, 1e-8f, bc1, bc2, weight_decay);
  return cudaGetLastError() == cudaSuccess ? HC_OK : HC_ERR_CUDA;
}

}  // extern "C"
