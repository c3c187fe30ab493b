// Small MLP for the learned Newton initial iterate: BF16 operands, FP32
// accumulation, hand-written tensor-core GEMM (warp MMA m16n8k16), forward,
// backward (MSE loss) and Adam, all on the device.
//
// Layout: every layer l maps K = size[l] inputs to N = size[l+1] outputs,
// Y = X W + b with W stored as W [K x N] and Wt [N x K] (both BF16, row-major)
// next to the FP32 master copy of Wt.  All dimensions are padded to multiples of
// 64 with zeros (padded weights, biases and activations stay exactly zero).
// Hidden layers use ReLU, the output layer is linear.
#include <cmath>
#include <cstring>
#include <cuda_bf16.h>
#include <random>
#include <vector>
#include "vfvm_context.cuh"

namespace vfvm {

constexpr int kTile = 64;   // CTA tile (M and N)
constexpr int kTileK = 32;  // K step

inline int pad64(int x) { return (x + 63) / 64 * 64; }

// C[M x N] (fp32) = A[M x K] . Bt[N x K]^T  (A, Bt bf16 row-major); M, N multiples
// of 64, K multiple of 32.  4 warps, each a 32 x 32 sub-tile of 2 x 4 MMAs.
// Epilogue (mode): 0 store C; 1 C + bias, relu -> Cout (fp32) and Cb (bf16);
// 2 C + bias -> Cout (fp32) and Cb (bf16).
__global__ void __launch_bounds__(128) gemm_bf16_kernel(int M, int N, int K, const __nv_bfloat16* __restrict__ A,
                                                        const __nv_bfloat16* __restrict__ Bt, float* __restrict__ C,
                                                        const float* __restrict__ bias, __nv_bfloat16* __restrict__ Cb,
                                                        int mode) {
  __shared__ __align__(16) __nv_bfloat16 sA[kTile][kTileK + 8];
  __shared__ __align__(16) __nv_bfloat16 sB[kTile][kTileK + 8];
  const int m0 = blockIdx.y * kTile, n0 = blockIdx.x * kTile;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
  const int g = lane >> 2, t = lane & 3;
  float acc[2][4][4];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int r = 0; r < 4; ++r) acc[i][j][r] = 0.f;
  for (int k0 = 0; k0 < K; k0 += kTileK) {
    // 64 rows x 32 bf16 = 64 x 4 chunks of 16 bytes per operand; 128 threads x 2 chunks
#pragma unroll
    for (int c = 0; c < 2; ++c) {
      const int idx = threadIdx.x + c * 128;
      const int row = idx >> 2, ch = (idx & 3) * 8;
      *reinterpret_cast<uint4*>(&sA[row][ch]) = *reinterpret_cast<const uint4*>(&A[(size_t)(m0 + row) * K + k0 + ch]);
      *reinterpret_cast<uint4*>(&sB[row][ch]) = *reinterpret_cast<const uint4*>(&Bt[(size_t)(n0 + row) * K + k0 + ch]);
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < kTileK; kk += 16) {
      uint32_t af[2][4], bf[4][2];
#pragma unroll
      for (int i = 0; i < 2; ++i) {
        const int r = wm + i * 16 + g;
        af[i][0] = *reinterpret_cast<const uint32_t*>(&sA[r][kk + 2 * t]);
        af[i][1] = *reinterpret_cast<const uint32_t*>(&sA[r + 8][kk + 2 * t]);
        af[i][2] = *reinterpret_cast<const uint32_t*>(&sA[r][kk + 2 * t + 8]);
        af[i][3] = *reinterpret_cast<const uint32_t*>(&sA[r + 8][kk + 2 * t + 8]);
      }
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int cidx = wn + j * 8 + g;
        bf[j][0] = *reinterpret_cast<const uint32_t*>(&sB[cidx][kk + 2 * t]);
        bf[j][1] = *reinterpret_cast<const uint32_t*>(&sB[cidx][kk + 2 * t + 8]);
      }
#pragma unroll
      for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
          asm volatile(
              "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
              "{%0,%1,%2,%3};\n"
              : "+f"(acc[i][j][0]), "+f"(acc[i][j][1]), "+f"(acc[i][j][2]), "+f"(acc[i][j][3])
              : "r"(af[i][0]), "r"(af[i][1]), "r"(af[i][2]), "r"(af[i][3]), "r"(bf[j][0]), "r"(bf[j][1]));
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int row = m0 + wm + i * 16 + g + 8 * h;
        const int col = n0 + wn + j * 8 + 2 * t;
#pragma unroll
        for (int e = 0; e < 2; ++e) {
          float v = acc[i][j][2 * h + e];
          if (mode >= 1) {
            v += bias[col + e];
            if (mode == 1) v = fmaxf(v, 0.f);
          }
          C[(size_t)row * N + col + e] = v;
          if (mode >= 1) Cb[(size_t)row * N + col + e] = __float2bfloat16_rn(v);
        }
      }
}

// out[c][r] = in[r][c] (bf16), rows x cols
__global__ void transpose_bf16_kernel(int rows, int cols, const __nv_bfloat16* __restrict__ in,
                                      __nv_bfloat16* __restrict__ out) {
  __shared__ __nv_bfloat16 tile[32][33];
  const int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
  for (int i = threadIdx.y; i < 32; i += blockDim.y) {
    const int r = r0 + i, c = c0 + threadIdx.x;
    if (r < rows && c < cols) tile[i][threadIdx.x] = in[(size_t)r * cols + c];
  }
  __syncthreads();
  for (int i = threadIdx.y; i < 32; i += blockDim.y) {
    const int c = c0 + i, r = r0 + threadIdx.x;
    if (r < rows && c < cols) out[(size_t)c * rows + r] = tile[threadIdx.x][i];
  }
}

// padded bf16 input from an fp32 [batch x k] array
__global__ void pack_input_kernel(int batch, int k, int Mp, int Kp, const float* __restrict__ X, __nv_bfloat16* __restrict__ Xb) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= (int64_t)Mp * Kp) return;
  const int r = (int)(i / Kp), c = (int)(i % Kp);
  Xb[i] = __float2bfloat16_rn((r < batch && c < k) ? X[(size_t)r * k + c] : 0.f);
}

// dY = 2 (Y - T) / (batch * n) on the valid block (bf16), loss partial sums
__global__ void mse_grad_kernel(int batch, int n, int Mp, int Np, const float* __restrict__ Y, const float* __restrict__ T,
                                __nv_bfloat16* __restrict__ dY, float* __restrict__ dYf, double* __restrict__ loss) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  double l = 0.0;
  if (i < (int64_t)Mp * Np) {
    const int r = (int)(i / Np), c = (int)(i % Np);
    float d = 0.f;
    if (r < batch && c < n) {
      const float e = Y[i] - T[(size_t)r * n + c];
      l = (double)e * e;
      d = 2.f * e / ((float)batch * (float)n);
    }
    dY[i] = __float2bfloat16_rn(d);
    dYf[i] = d;
  }
  for (int o = 16; o > 0; o >>= 1) l += __shfl_down_sync(0xffffffffu, l, o);
  if ((threadIdx.x & 31) == 0 && l != 0.0) atomicAdd(loss, l);
}

// dZ = dA * relu'(Z) (in place on the fp32 copy), bf16 copy
__global__ void relu_grad_kernel(int64_t n, const float* __restrict__ Z, float* __restrict__ dA, __nv_bfloat16* __restrict__ dZb) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float d = Z[i] > 0.f ? dA[i] : 0.f;
  dA[i] = d;
  dZb[i] = __float2bfloat16_rn(d);
}

// db[n] = sum_m dZ[m][n]
__global__ void bias_grad_kernel(int Mp, int Np, const float* __restrict__ dZ, float* __restrict__ db) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= Np) return;
  float s = 0.f;
  for (int r = 0; r < Mp; ++r) s += dZ[(size_t)r * Np + c];
  db[c] = s;
}

// Adam on the fp32 master Wt and b; refresh the bf16 copies Wt (N x K) and W (K x N)
__global__ void adam_kernel(int64_t n, float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                            float* __restrict__ v, float lr, float b1, float b2, float eps, float c1, float c2) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

__global__ void refresh_bf16_kernel(int Np, int Kp, const float* __restrict__ Wt, __nv_bfloat16* __restrict__ Wtb,
                                    __nv_bfloat16* __restrict__ Wb) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= (int64_t)Np * Kp) return;
  const int n = (int)(i / Kp), k = (int)(i % Kp);
  const __nv_bfloat16 w = __float2bfloat16_rn(Wt[i]);
  Wtb[i] = w;
  Wb[(size_t)k * Np + n] = w;
}

__global__ void unpack_output_kernel(int batch, int n, int Np, const float* __restrict__ Y, float* __restrict__ out) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= (int64_t)batch * n) return;
  out[i] = Y[(size_t)(i / n) * Np + i % n];
}

}  // namespace vfvm

using namespace vfvm;

struct vfvm_mlp {
  int L = 0, max_batch = 0, Mp = 0;
  std::vector<int> size, psize;
  std::vector<DBuf<float>*> Wt, b, gWt, gb, mW, vW, mb, vb;   // fp32 master, grads, Adam moments
  std::vector<DBuf<__nv_bfloat16>*> Wtb, Wb;                 // bf16 copies
  std::vector<DBuf<__nv_bfloat16>*> Xb, XTb;                 // layer inputs (bf16) and transposes
  std::vector<DBuf<float>*> Z;                               // pre/post activation (fp32)
  DBuf<__nv_bfloat16> dZb, dZTb;
  DBuf<float> dA;
  DBuf<double> loss;
  int step = 0;
  cudaStream_t stream = nullptr;
  ~vfvm_mlp() {
    for (auto* v : {&Wt, &b, &gWt, &gb, &mW, &vW, &mb, &vb, &Z})
      for (auto* p : *v) delete p;
    for (auto* v : {&Wtb, &Wb, &Xb, &XTb})
      for (auto* p : *v) delete p;
    if (stream) cudaStreamDestroy(stream);
  }
};

namespace {

template <class T>
DBuf<T>* newbuf(size_t n, cudaError_t& e) {
  auto* d = new DBuf<T>;
  if (e == cudaSuccess) e = d->alloc(n);
  if (e == cudaSuccess && n) e = cudaMemset(d->p, 0, n * sizeof(T));
  return d;
}

inline unsigned nb(int64_t n, int t = 256) { return (unsigned)((n + t - 1) / t); }

int gemm(vfvm_mlp* m, int M, int N, int K, const __nv_bfloat16* A, const __nv_bfloat16* Bt, float* C, const float* bias,
         __nv_bfloat16* Cb, int mode) {
  if (M % kTile || N % kTile || K % kTileK) return VFVM_ERR_INPUT;
  dim3 grid(N / kTile, M / kTile);
  gemm_bf16_kernel<<<grid, 128, 0, m->stream>>>(M, N, K, A, Bt, C, bias, Cb, mode);
  VFVM_CUDA(cudaGetLastError());
  return VFVM_OK;
}

int forward(vfvm_mlp* m, int batch, const float* X) {
  const int Mp = m->Mp;
  pack_input_kernel<<<nb((int64_t)Mp * m->psize[0]), 256, 0, m->stream>>>(batch, m->size[0], Mp, m->psize[0], X, m->Xb[0]->p);
  for (int l = 0; l < m->L; ++l) {
    const int K = m->psize[l], N = m->psize[l + 1];
    const int mode = (l + 1 < m->L) ? 1 : 2;
    int rc = gemm(m, Mp, N, K, m->Xb[l]->p, m->Wtb[l]->p, m->Z[l]->p, m->b[l]->p, m->Xb[l + 1]->p, mode);
    if (rc) return rc;
  }
  return VFVM_OK;
}

// gradients of the MSE loss into gWt/gb; loss (mean) into *loss_out
int backward(vfvm_mlp* m, int batch, const float* T, float* loss_out) {
  const int Mp = m->Mp, L = m->L;
  VFVM_CUDA(cudaMemsetAsync(m->loss.p, 0, sizeof(double), m->stream));
  const int No = m->psize[L];
  mse_grad_kernel<<<nb((int64_t)Mp * No), 256, 0, m->stream>>>(batch, m->size[L], Mp, No, m->Z[L - 1]->p, T, m->dZb.p,
                                                                m->dA.p, m->loss.p);
  for (int l = L - 1; l >= 0; --l) {
    const int K = m->psize[l], N = m->psize[l + 1];
    if (l + 1 < L)  // hidden layer: dZ = dA * relu'(Z)
      relu_grad_kernel<<<nb((int64_t)Mp * N), 256, 0, m->stream>>>((int64_t)Mp * N, m->Z[l]->p, m->dA.p, m->dZb.p);
    // dWt[N x K] = dZ^T [N x M] . X [M x K]  ->  A = dZ^T, Bt = X^T
    transpose_bf16_kernel<<<dim3(nb(N, 32), nb(Mp, 32)), dim3(32, 8), 0, m->stream>>>(Mp, N, m->dZb.p, m->dZTb.p);
    transpose_bf16_kernel<<<dim3(nb(K, 32), nb(Mp, 32)), dim3(32, 8), 0, m->stream>>>(Mp, K, m->Xb[l]->p, m->XTb[l]->p);
    int rc = gemm(m, N, K, Mp, m->dZTb.p, m->XTb[l]->p, m->gWt[l]->p, nullptr, nullptr, 0);
    if (rc) return rc;
    bias_grad_kernel<<<nb(N), 256, 0, m->stream>>>(Mp, N, m->dA.p, m->gb[l]->p);
    if (l > 0) {  // dA_prev [M x K] = dZ [M x N] . W^T  ->  Bt = W [K x N]
      rc = gemm(m, Mp, K, N, m->dZb.p, m->Wb[l]->p, m->dA.p, nullptr, nullptr, 0);
      if (rc) return rc;
    }
  }
  if (loss_out) {  // reading the loss waits for the step; without it the steps queue up
    double h = 0.0;
    VFVM_CUDA(cudaMemcpyAsync(&h, m->loss.p, sizeof(double), cudaMemcpyDeviceToHost, m->stream));
    VFVM_CUDA(cudaStreamSynchronize(m->stream));
    *loss_out = (float)(h / ((double)batch * m->size[L]));
  }
  return VFVM_OK;
}

}  // namespace

extern "C" vfvm_mlp* vfvm_mlp_create(int32_t nlayers, const int32_t* sizes, int32_t max_batch, uint64_t seed,
                                     int* status) {
  int dummy;
  if (!status) status = &dummy;
  *status = VFVM_ERR_INPUT;
  if (nlayers < 1 || nlayers > 16 || !sizes || max_batch < 1) return nullptr;
  for (int l = 0; l <= nlayers; ++l) if (sizes[l] < 1 || sizes[l] > 8192) return nullptr;
  vfvm_mlp* m = new vfvm_mlp;
  m->L = nlayers;
  m->max_batch = max_batch;
  m->Mp = pad64(max_batch);
  int maxp = 0;
  for (int l = 0; l <= nlayers; ++l) {
    m->size.push_back(sizes[l]);
    m->psize.push_back(pad64(sizes[l]));
    maxp = std::max(maxp, m->psize.back());
  }
  // a blocking stream: work queued on the legacy default stream before a call
  // (inputs written by the caller) completes before the network reads it
  cudaError_t e = cudaStreamCreate(&m->stream);
  std::mt19937_64 rng(seed);
  for (int l = 0; l < nlayers; ++l) {
    const int K = m->psize[l], N = m->psize[l + 1];
    const size_t nw = (size_t)N * K;
    m->Wt.push_back(newbuf<float>(nw, e)); m->b.push_back(newbuf<float>(N, e));
    m->gWt.push_back(newbuf<float>(nw, e)); m->gb.push_back(newbuf<float>(N, e));
    m->mW.push_back(newbuf<float>(nw, e)); m->vW.push_back(newbuf<float>(nw, e));
    m->mb.push_back(newbuf<float>(N, e)); m->vb.push_back(newbuf<float>(N, e));
    m->Wtb.push_back(newbuf<__nv_bfloat16>(nw, e)); m->Wb.push_back(newbuf<__nv_bfloat16>(nw, e));
    m->Z.push_back(newbuf<float>((size_t)m->Mp * N, e));
    // He initialisation on the valid block, zeros in the padding
    std::vector<float> w(nw, 0.f);
    std::normal_distribution<float> nd(0.f, std::sqrt(2.f / (float)sizes[l]));
    for (int n = 0; n < sizes[l + 1]; ++n)
      for (int k = 0; k < sizes[l]; ++k) w[(size_t)n * K + k] = nd(rng);
    if (e == cudaSuccess) e = cudaMemcpy(m->Wt[l]->p, w.data(), nw * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
      refresh_bf16_kernel<<<nb((int64_t)nw), 256, 0, m->stream>>>(N, K, m->Wt[l]->p, m->Wtb[l]->p, m->Wb[l]->p);
      e = cudaGetLastError();
    }
  }
  for (int l = 0; l <= nlayers; ++l) {
    m->Xb.push_back(newbuf<__nv_bfloat16>((size_t)m->Mp * m->psize[l], e));
    m->XTb.push_back(newbuf<__nv_bfloat16>((size_t)m->Mp * m->psize[l], e));
  }
  m->dZb.n = 0;
  if (e == cudaSuccess) e = m->dZb.alloc((size_t)m->Mp * maxp);
  if (e == cudaSuccess) e = m->dZTb.alloc((size_t)m->Mp * maxp);
  if (e == cudaSuccess) e = m->dA.alloc((size_t)m->Mp * maxp);
  if (e == cudaSuccess) e = m->loss.alloc(1);
  if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
  if (e != cudaSuccess) {
    fprintf(stderr, "vfvm_mlp_create: %s\n", cudaGetErrorString(e));
    *status = VFVM_ERR_CUDA;
    delete m;
    return nullptr;
  }
  *status = VFVM_OK;
  return m;
}

extern "C" void vfvm_mlp_destroy(vfvm_mlp* m) { delete m; }

extern "C" int vfvm_mlp_nparams(vfvm_mlp* m, int64_t* n) {
  if (!m || !n) return VFVM_ERR_INPUT;
  int64_t s = 0;
  for (int l = 0; l < m->L; ++l) s += (int64_t)m->size[l] * m->size[l + 1] + m->size[l + 1];
  *n = s;
  return VFVM_OK;
}

// Parameters in the order W0 [K0 x N0] row-major, b0 [N0], W1, b1, ... (fp32, host).
// out != NULL: read them; in != NULL: replace them (then the bf16 copies are refreshed).
extern "C" int vfvm_mlp_params(vfvm_mlp* m, float* out, const float* in) {
  if (!m) return VFVM_ERR_INPUT;
  VFVM_CUDA(cudaStreamSynchronize(m->stream));
  size_t off = 0;
  for (int l = 0; l < m->L; ++l) {
    const int K = m->psize[l], N = m->psize[l + 1], k = m->size[l], n = m->size[l + 1];
    std::vector<float> wt((size_t)N * K), bb(N);
    VFVM_CUDA(cudaMemcpy(wt.data(), m->Wt[l]->p, wt.size() * sizeof(float), cudaMemcpyDeviceToHost));
    VFVM_CUDA(cudaMemcpy(bb.data(), m->b[l]->p, bb.size() * sizeof(float), cudaMemcpyDeviceToHost));
    if (out) {
      for (int kk = 0; kk < k; ++kk)
        for (int nn = 0; nn < n; ++nn) out[off + (size_t)kk * n + nn] = wt[(size_t)nn * K + kk];
      for (int nn = 0; nn < n; ++nn) out[off + (size_t)k * n + nn] = bb[nn];
    }
    if (in) {
      for (int kk = 0; kk < k; ++kk)
        for (int nn = 0; nn < n; ++nn) wt[(size_t)nn * K + kk] = in[off + (size_t)kk * n + nn];
      for (int nn = 0; nn < n; ++nn) bb[nn] = in[off + (size_t)k * n + nn];
      VFVM_CUDA(cudaMemcpy(m->Wt[l]->p, wt.data(), wt.size() * sizeof(float), cudaMemcpyHostToDevice));
      VFVM_CUDA(cudaMemcpy(m->b[l]->p, bb.data(), bb.size() * sizeof(float), cudaMemcpyHostToDevice));
      refresh_bf16_kernel<<<nb((int64_t)N * K), 256, 0, m->stream>>>(N, K, m->Wt[l]->p, m->Wtb[l]->p, m->Wb[l]->p);
      VFVM_CUDA(cudaGetLastError());
    }
    off += (size_t)k * n + n;
  }
  VFVM_CUDA(cudaStreamSynchronize(m->stream));
  return VFVM_OK;
}

// Y [batch x out] = net(X [batch x in]); X, Y fp32 device pointers.
extern "C" int vfvm_mlp_forward(vfvm_mlp* m, int32_t batch, const float* X, float* Y) {
  if (!m || batch < 1 || batch > m->max_batch || !X || !Y) return VFVM_ERR_INPUT;
  int rc = forward(m, batch, X);
  if (rc) return rc;
  const int n = m->size[m->L];
  unpack_output_kernel<<<nb((int64_t)batch * n), 256, 0, m->stream>>>(batch, n, m->psize[m->L], m->Z[m->L - 1]->p, Y);
  VFVM_CUDA(cudaGetLastError());
  VFVM_CUDA(cudaStreamSynchronize(m->stream));
  return VFVM_OK;
}

// Gradients of the mean squared error of net(X) against T (device inputs) in the
// vfvm_mlp_params order (host), and the loss.
extern "C" int vfvm_mlp_gradients(vfvm_mlp* m, int32_t batch, const float* X, const float* T, float* grads,
                                  float* loss) {
  if (!m || batch < 1 || batch > m->max_batch || !X || !T) return VFVM_ERR_INPUT;
  int rc = forward(m, batch, X);
  if (rc) return rc;
  if ((rc = backward(m, batch, T, loss))) return rc;
  VFVM_CUDA(cudaStreamSynchronize(m->stream));
  if (grads) {
    size_t off = 0;
    for (int l = 0; l < m->L; ++l) {
      const int K = m->psize[l], N = m->psize[l + 1], k = m->size[l], n = m->size[l + 1];
      std::vector<float> g((size_t)N * K), gb(N);
      VFVM_CUDA(cudaMemcpy(g.data(), m->gWt[l]->p, g.size() * sizeof(float), cudaMemcpyDeviceToHost));
      VFVM_CUDA(cudaMemcpy(gb.data(), m->gb[l]->p, gb.size() * sizeof(float), cudaMemcpyDeviceToHost));
      for (int kk = 0; kk < k; ++kk)
        for (int nn = 0; nn < n; ++nn) grads[off + (size_t)kk * n + nn] = g[(size_t)nn * K + kk];
      for (int nn = 0; nn < n; ++nn) grads[off + (size_t)k * n + nn] = gb[nn];
      off += (size_t)k * n + n;
    }
  }
  return VFVM_OK;
}

// One Adam step (lr, beta1 0.9, beta2 0.999, eps 1e-8) on the MSE loss of a batch.
extern "C" int vfvm_mlp_train_step(vfvm_mlp* m, int32_t batch, const float* X, const float* T, float lr, float* loss) {
  if (!m || batch < 1 || batch > m->max_batch || !X || !T || !(lr > 0)) return VFVM_ERR_INPUT;
  int rc = forward(m, batch, X);
  if (rc) return rc;
  if ((rc = backward(m, batch, T, loss))) return rc;
  m->step += 1;
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.f - std::pow(b1, (float)m->step), c2 = 1.f - std::pow(b2, (float)m->step);
  for (int l = 0; l < m->L; ++l) {
    const int K = m->psize[l], N = m->psize[l + 1];
    const int64_t nw = (int64_t)N * K;
    adam_kernel<<<nb(nw), 256, 0, m->stream>>>(nw, m->Wt[l]->p, m->gWt[l]->p, m->mW[l]->p, m->vW[l]->p, lr, b1, b2, 1e-8f, c1, c2);
    adam_kernel<<<nb(N), 256, 0, m->stream>>>(N, m->b[l]->p, m->gb[l]->p, m->mb[l]->p, m->vb[l]->p, lr, b1, b2, 1e-8f, c1, c2);
    refresh_bf16_kernel<<<nb(nw), 256, 0, m->stream>>>(N, K, m->Wt[l]->p, m->Wtb[l]->p, m->Wb[l]->p);
  }
  VFVM_CUDA(cudaGetLastError());
  return VFVM_OK;
}

namespace vfvm {

// fine[b][ix + nf*iy] = s_b * (scale * (bilinear interpolation of coarse[b][cx + nc*cy]) + shift),
// nf = (nc-1)*r+1, s_b = inst_scale[b] (1 without inst_scale)
__global__ void prolong_bilinear_kernel(int batch, int nc, int r, const float* __restrict__ coarse, int64_t cstride,
                                        double scale, double shift, const double* __restrict__ inst_scale,
                                        double* __restrict__ fine, int64_t fstride) {
  const int nf = (nc - 1) * r + 1;
  const int64_t per = (int64_t)nf * nf;
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= per * batch) return;
  const int b = (int)(i / per);
  const int k = (int)(i % per);
  const int ix = k % nf, iy = k / nf;
  const int cx = min(ix / r, nc - 2), cy = min(iy / r, nc - 2);
  const double tx = (double)(ix - cx * r) / r, ty = (double)(iy - cy * r) / r;
  const float* c = coarse + b * cstride + cx + (int64_t)nc * cy;
  const double v = (1.0 - tx) * (1.0 - ty) * c[0] + tx * (1.0 - ty) * c[1] + (1.0 - tx) * ty * c[nc] + tx * ty * c[nc + 1];
  fine[b * fstride + k] = (inst_scale ? inst_scale[b] : 1.0) * (scale * v + shift);
}

}  // namespace vfvm

// Bilinear prolongation of batch coarse fields (nc x nc nodes, x fastest, FP32),
// times scale plus shift, times an optional per-instance factor, onto the nested fine grids ((nc-1)*ratio+1 nodes per side, FP64), e.g. a
// coarse network prediction to a Newton initial value.  Device pointers; the
// instance b reads coarse + b*coarse_stride and writes fine + b*fine_stride.
extern "C" int vfvm_prolong_bilinear(int32_t batch, int32_t nc, int32_t ratio, const float* coarse,
                                     int64_t coarse_stride, double scale, double shift, const double* inst_scale,
                                     double* fine, int64_t fine_stride, void* stream) {
  if (batch < 1 || nc < 2 || ratio < 1 || !coarse || !fine) return VFVM_ERR_INPUT;
  const int64_t nf = (int64_t)(nc - 1) * ratio + 1;
  if (coarse_stride < (int64_t)nc * nc || fine_stride < nf * nf) return VFVM_ERR_INPUT;
  const int64_t total = nf * nf * batch;
  prolong_bilinear_kernel<<<nb(total), 256, 0, (cudaStream_t)stream>>>(batch, nc, ratio, coarse, coarse_stride, scale,
                                                                       shift, inst_scale, fine, fine_stride);
  VFVM_CUDA(cudaGetLastError());
  return VFVM_OK;
}

namespace vfvm {

// X[b][c] = mean of log(field[b][k]) over the fine nodes k of the window of
// half-width `half` around coarse node c (clipped at the boundary; half = 0:
// the node itself), c = cx + nc*cy at fine node (cx*r, cy*r); X[b][nc*nc] = extra[b]
__global__ void coarse_log_features_kernel(int batch, int nc, int r, int half, const double* __restrict__ field,
                                           int64_t fstride, const double* __restrict__ extra, float* __restrict__ X) {
  const int nf = (nc - 1) * r + 1;
  const int nin = nc * nc + 1;
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= (int64_t)batch * nin) return;
  const int b = (int)(i / nin), c = (int)(i % nin);
  if (c == nc * nc) {
    X[i] = extra ? (float)extra[b] : 0.0f;
    return;
  }
  const int cx = c % nc, cy = c / nc;
  const int x0 = max(cx * r - half, 0), x1 = min(cx * r + half, nf - 1);
  const int y0 = max(cy * r - half, 0), y1 = min(cy * r + half, nf - 1);
  const double* F = field + b * fstride;
  double s = 0.0;
  for (int y = y0; y <= y1; ++y)
    for (int x = x0; x <= x1; ++x) s += ::log(F[x + (int64_t)nf * y]);
  X[i] = (float)(s / ((x1 - x0 + 1) * (y1 - y0 + 1)));
}

}  // namespace vfvm

// Network input features of a batch of positive node fields (e.g. the kappa of
// the kappa_exp instances) on nested square grids: the mean of log(field) over
// a (2 half + 1)^2 window around each node of the nc x nc coarse subgrid (every
// ratio-th fine node; half = 0 takes the node's own value), then one extra
// scalar per instance (e.g. the source f).  Device pointers; X is FP32, batch
// rows of nc*nc + 1 values; enqueued on stream (NULL: the legacy default stream).
extern "C" int vfvm_coarse_log_features(int32_t batch, int32_t nc, int32_t ratio, int32_t half, const double* field,
                                        int64_t field_stride, const double* extra, float* X, void* stream) {
  if (batch < 1 || nc < 2 || ratio < 1 || half < 0 || half > ratio || !field || !X) return VFVM_ERR_INPUT;
  const int64_t nf = (int64_t)(nc - 1) * ratio + 1;
  if (field_stride < nf * nf) return VFVM_ERR_INPUT;
  const int64_t total = (int64_t)batch * (nc * nc + 1);
  coarse_log_features_kernel<<<nb(total), 256, 0, (cudaStream_t)stream>>>(batch, nc, ratio, half, field, field_stride,
                                                                         extra, X);
  VFVM_CUDA(cudaGetLastError());
  return VFVM_OK;
}
