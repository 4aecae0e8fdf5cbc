// Learned force closure: a small 3D CNN on the PM mesh that predicts the
// residual between the force of a finer mesh and the mesh force, trained on
// the GPU by the kernels of this file (no counterpart in the reference).
//
// Network: four periodic 3x3x3 convolutions, 16 channels between layers,
// ReLU after the first three, the last layer linear with 3 outputs (the
// residual force components).  Inputs per cell (padded to 16 channels):
// asinh(delta), asinh(Phi_N / 1e-5) and the screening factor
// min(1, |phi_crit / Phi_N|) for Phi_N < 0 (1 otherwise, and 1 for models
// without potential screening).  Activations and weights are BF16, every
// accumulation is FP32 on the tensor cores (mma.sync m16n8k16 bf16).
//
// Layout: activations channel-last [V][16] bf16 with voxel v = (i N + j) N + k
// (k fastest, as the mesh rows); weights [27 taps][16 out][16 in], tap =
// 9 (di+1) + 3 (dj+1) + (dk+1) for offsets d in {-1, 0, 1}.
//
// Convolution as implicit GEMM: a block takes 64 consecutive voxels of one
// (i, j) row; it stages the 9 neighbouring rows (i+di, j+dj), each with one
// halo voxel on either side, and all weights in shared memory; warp w owns
// 16 voxels and runs, for each tap, one 16x16x16 product as two m16n8k16
// MMAs whose A fragment is the 16 voxels shifted by dk (ldmatrix), so every
// staged row serves the three dk taps.  The data gradient is the same
// convolution with the weights mirrored (tap -> 26 - tap) and transposed
// (in <-> out); the weight gradient is, per tap, dY^T X over all voxels,
// accumulated by persistent blocks in registers and reduced with one FP32
// atomic per weight per block.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <vector>

#include "mgp_internal.h"

typedef __nv_bfloat16 bf16;

#define NN_CH 16
#define NN_TAPS 27
#define NN_LAYERS 4
#define NN_SEG 64
#define NN_WSIZE (NN_TAPS * NN_CH * NN_CH)

struct mgp_closure {
  int N;
  long long V;
  int device;
  cudaStream_t stream;
  int own_stream;
  float *w32[NN_LAYERS], *b32[NN_LAYERS];  // FP32 master weights
  float *gw[NN_LAYERS], *gb[NN_LAYERS];    // gradients
  float *mw[NN_LAYERS], *vw[NN_LAYERS], *mb[NN_LAYERS], *vb[NN_LAYERS];  // Adam moments
  bf16 *w16[NN_LAYERS];                    // BF16 copies, forward layout
  bf16 *wt16;                              // mirrored + transposed scratch
  int adam_t;
  bf16 *act[NN_LAYERS];                    // act[0] = features, act[l] = output of layer l
  float *out;                              // last layer output [V][4]
  float *target;                           // [V][4]
  bf16 *g0, *g1;                           // gradient ping-pong [V][16]
  double *loss;                            // device scalar
  float out_scale;                         // residual = out_scale * network output
  float *grid_a, *grid_b;                  // scratch real grids for the features
  long long P;                             // padded row of the scratch grids
  // stored training samples: features (3 bf16) and targets (3 f32) per voxel
  int nsamples, cap_samples;
  bf16 *ds_x;
  float *ds_t;
};

namespace {

constexpr int kThreadsConv = 128;  // 4 warps x 16 voxels = NN_SEG
constexpr int kThreadsWg = 256;

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void ldsm_x4(uint32_t addr, uint32_t &r0, uint32_t &r1, uint32_t &r2, uint32_t &r3) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
               : "r"(addr));
}
__device__ __forceinline__ void ldsm_x4_t(uint32_t addr, uint32_t &r0, uint32_t &r1, uint32_t &r2, uint32_t &r3) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
               : "r"(addr));
}
__device__ __forceinline__ void mma16816(float (&d)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3,
                                         uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// Stage the 9 rows (i+di, j+dj), voxels k0-1 .. k0+NN_SEG (periodic), of a
// [V][16] bf16 tensor: xs[r][q] with r = 3 (di+1) + (dj+1), q = voxel - (k0-1).
// A segment that ends before k0+NN_SEG (N not a multiple of NN_SEG) stages
// voxels k0-1 .. N (the last one wraps to 0) and zeros after them, so every
// read stays inside the tensor.
__device__ __forceinline__ void stage_rows(const bf16 *__restrict__ X, int N, int i, int j, int k0,
                                           bf16 (*xs)[NN_SEG + 2][NN_CH], int tid, int nthr) {
  const int per_row = (NN_SEG + 2) * 2;  // 16-byte chunks per staged row
  const int qmax = min(NN_SEG + 1, N - k0 + 1);
  for (int c = tid; c < 9 * per_row; c += nthr) {
    const int r = c / per_row, q = (c % per_row) >> 1, h = c & 1;
    if (q > qmax) {
      reinterpret_cast<uint4 *>(&xs[r][q][0])[h] = make_uint4(0, 0, 0, 0);
      continue;
    }
    int ii = i + r / 3 - 1, jj = j + r % 3 - 1, kk = k0 - 1 + q;
    ii += ii < 0 ? N : 0;
    ii -= ii >= N ? N : 0;
    jj += jj < 0 ? N : 0;
    jj -= jj >= N ? N : 0;
    kk += kk < 0 ? N : 0;
    kk -= kk >= N ? N : 0;
    const long long v = ((long long)ii * N + jj) * N + kk;
    reinterpret_cast<uint4 *>(&xs[r][q][0])[h] = reinterpret_cast<const uint4 *>(X + v * NN_CH)[h];
  }
}

// Forward convolution.  mode 0: bf16 out, bias + ReLU; 1: bf16 out, no bias
// (data gradient); 2: f32 out [V][4] (channels 0-3), bias; 3: add
// scale * (out + bias) to the three force grids (channels 0-2).
__global__ void __launch_bounds__(kThreadsConv) k_conv_fwd(const bf16 *__restrict__ X, const bf16 *__restrict__ W,
                                                           const float *__restrict__ bias, int N, int mode,
                                                           bf16 *__restrict__ Y16, float *__restrict__ Y32,
                                                           float *__restrict__ frc, long long gstride, long long P,
                                                           float scale) {
  __shared__ __align__(16) bf16 ws[NN_WSIZE];
  __shared__ __align__(16) bf16 xs[9][NN_SEG + 2][NN_CH];
  const int nseg = (N + NN_SEG - 1) / NN_SEG;
  const long long row = blockIdx.x / nseg;
  const int seg = (int)(blockIdx.x - row * nseg);
  const int i = (int)(row / N), j = (int)(row - (long long)i * N), k0 = seg * NN_SEG;
  const int tid = threadIdx.x;
  for (int c = tid; c < NN_WSIZE / 8; c += kThreadsConv)
    reinterpret_cast<uint4 *>(ws)[c] = reinterpret_cast<const uint4 *>(W)[c];
  stage_rows(X, N, i, j, k0, xs, tid, kThreadsConv);
  __syncthreads();
  const int warp = tid >> 5, lane = tid & 31;
  const int kw = k0 + 16 * warp;  // first voxel of this warp
  if (kw >= N) return;
  float acc0[4] = {0.f, 0.f, 0.f, 0.f}, acc1[4] = {0.f, 0.f, 0.f, 0.f};
  // ldmatrix lane roles: A (16 voxels x 16 ch), B (16 out x 16 in)
  const int a_vox = (lane & 7) + 8 * ((lane >> 3) & 1), a_half = lane >> 4;
  const int b_out = (lane & 7) + 8 * (lane >> 4), b_half = (lane >> 3) & 1;
#pragma unroll 1
  for (int tap = 0; tap < NN_TAPS; tap++) {
    const int r = tap / 3, dk = tap % 3;
    uint32_t a0, a1, a2, a3, b0, b1, b2, b3;
    ldsm_x4(smem_u32(&xs[r][16 * warp + dk + a_vox][8 * a_half]), a0, a1, a2, a3);
    ldsm_x4(smem_u32(&ws[(tap * NN_CH + b_out) * NN_CH + 8 * b_half]), b0, b1, b2, b3);
    mma16816(acc0, a0, a1, a2, a3, b0, b1);
    mma16816(acc1, a0, a1, a2, a3, b2, b3);
  }
  // fragment: rows (voxels) lane/4 and lane/4 + 8, columns 2 (lane%4) + {0,1}
  const int vr = lane >> 2, cc = 2 * (lane & 3);
  const long long vb = ((long long)i * N + j) * N + kw;
#pragma unroll
  for (int h = 0; h < 2; h++) {
    const long long v = vb + vr + 8 * h;
    float o[4] = {acc0[2 * h], acc0[2 * h + 1], acc1[2 * h], acc1[2 * h + 1]};  // ch cc, cc+1, cc+8, cc+9
    if (mode != 1 && bias) {
      o[0] += bias[cc];
      o[1] += bias[cc + 1];
      o[2] += bias[cc + 8];
      o[3] += bias[cc + 9];
    }
    if (mode <= 1) {
      if (mode == 0)
#pragma unroll
        for (int q = 0; q < 4; q++) o[q] = fmaxf(o[q], 0.f);
      reinterpret_cast<__nv_bfloat162 *>(Y16 + v * NN_CH + cc)[0] = __floats2bfloat162_rn(o[0], o[1]);
      reinterpret_cast<__nv_bfloat162 *>(Y16 + v * NN_CH + cc + 8)[0] = __floats2bfloat162_rn(o[2], o[3]);
    } else if (cc < 4) {
      if (mode == 2) {
        Y32[v * 4 + cc] = o[0];
        Y32[v * 4 + cc + 1] = o[1];
      } else {
        const int kk = kw + vr + 8 * h;
        const long long g = ((long long)i * N + j) * P + kk;
        frc[cc * gstride + g] += scale * o[0];
        if (cc + 1 < 3) frc[(cc + 1) * gstride + g] += scale * o[1];
      }
    }
  }
}

// Weight and bias gradients: dW[tap][o][c] += sum_v dY[v][o] X[v + d(tap)][c],
// db[o] += sum_v dY[v][o]; persistent blocks over (row, segment) units.
__global__ void __launch_bounds__(kThreadsWg) k_conv_wgrad(const bf16 *__restrict__ X, const bf16 *__restrict__ dY,
                                                           int N, float *__restrict__ dW, float *__restrict__ db) {
  __shared__ __align__(16) bf16 xs[9][NN_SEG + 2][NN_CH];
  __shared__ __align__(16) bf16 ys[NN_SEG][NN_CH];
  const int nseg = (N + NN_SEG - 1) / NN_SEG;
  const long long units = (long long)N * N * nseg;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  float acc[4][2][4];
#pragma unroll
  for (int t = 0; t < 4; t++)
#pragma unroll
    for (int n = 0; n < 2; n++)
#pragma unroll
      for (int q = 0; q < 4; q++) acc[t][n][q] = 0.f;
  float bacc = 0.f;
  // ldmatrix.trans lane roles: A = dY^T (16 out x 16 voxels), B = X (16 voxels x 16 in)
  const int a_vox = (lane & 7) + 8 * (lane >> 4), a_half = (lane >> 3) & 1;
  const int b_vox = (lane & 7) + 8 * ((lane >> 3) & 1), b_half = lane >> 4;
  for (long long u = blockIdx.x; u < units; u += gridDim.x) {
    const long long row = u / nseg;
    const int seg = (int)(u - row * nseg);
    const int i = (int)(row / N), j = (int)(row - (long long)i * N), k0 = seg * NN_SEG;
    __syncthreads();
    stage_rows(X, N, i, j, k0, xs, tid, kThreadsWg);
    for (int c = tid; c < NN_SEG * 2; c += kThreadsWg) {
      const int q = c >> 1, h = c & 1, kk = k0 + q;
      uint4 val = make_uint4(0, 0, 0, 0);
      if (kk < N) val = reinterpret_cast<const uint4 *>(dY + (((long long)i * N + j) * N + kk) * NN_CH)[h];
      reinterpret_cast<uint4 *>(&ys[q][0])[h] = val;
    }
    __syncthreads();
    if (tid < NN_CH)
      for (int q = 0; q < NN_SEG; q++) bacc += __bfloat162float(ys[q][tid]);
#pragma unroll
    for (int t = 0; t < 4; t++) {
      const int tap = warp + 8 * t;
      if (tap >= NN_TAPS) break;
      const int r = tap / 3, dk = tap % 3;
#pragma unroll
      for (int ks = 0; ks < NN_SEG / 16; ks++) {
        uint32_t a0, a1, a2, a3, b0, b1, b2, b3;
        ldsm_x4_t(smem_u32(&ys[16 * ks + a_vox][8 * a_half]), a0, a1, a2, a3);
        ldsm_x4_t(smem_u32(&xs[r][16 * ks + dk + b_vox][8 * b_half]), b0, b1, b2, b3);
        mma16816(acc[t][0], a0, a1, a2, a3, b0, b1);
        mma16816(acc[t][1], a0, a1, a2, a3, b2, b3);
      }
    }
  }
  // fragment: rows (out) lane/4, lane/4 + 8; columns (in) 2 (lane%4) + {0,1} (+8 for n-tile 1)
  const int o0 = lane >> 2, c0 = 2 * (lane & 3);
#pragma unroll
  for (int t = 0; t < 4; t++) {
    const int tap = warp + 8 * t;
    if (tap >= NN_TAPS) break;
    float *w = dW + tap * NN_CH * NN_CH;
#pragma unroll
    for (int n = 0; n < 2; n++) {
      atomicAdd(w + o0 * NN_CH + c0 + 8 * n, acc[t][n][0]);
      atomicAdd(w + o0 * NN_CH + c0 + 8 * n + 1, acc[t][n][1]);
      atomicAdd(w + (o0 + 8) * NN_CH + c0 + 8 * n, acc[t][n][2]);
      atomicAdd(w + (o0 + 8) * NN_CH + c0 + 8 * n + 1, acc[t][n][3]);
    }
  }
  if (tid < NN_CH) atomicAdd(db + tid, bacc);
}

// dY *= relu'(Y) (Y the layer's bf16 output)
__global__ void k_relu_grad(bf16 *__restrict__ dY, const bf16 *__restrict__ Y, long long n) {
  long long stride = (long long)gridDim.x * blockDim.x;
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += stride)
    if (!(__bfloat162float(Y[q]) > 0.f)) dY[q] = __float2bfloat16_rn(0.f);
}

// Wt[26 - tap][c][o] = W[tap][o][c]
__global__ void k_mirror_transpose(const bf16 *__restrict__ W, bf16 *__restrict__ Wt) {
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < NN_WSIZE; q += gridDim.x * blockDim.x) {
    const int tap = q / (NN_CH * NN_CH), o = (q / NN_CH) % NN_CH, c = q % NN_CH;
    Wt[((NN_TAPS - 1 - tap) * NN_CH + c) * NN_CH + o] = W[q];
  }
}

// MSE over the 3 residual components, loss = sum (s out - t)^2 / (3 V) with
// s = out_scale; dOut (bf16, channels 0-2, zero elsewhere) = d loss / d out.
__global__ void k_loss_grad(const float *__restrict__ out, const float *__restrict__ tgt, long long V, float s,
                            bf16 *__restrict__ g, double *__restrict__ loss) {
  __shared__ double sh[8];
  long long stride = (long long)gridDim.x * blockDim.x;
  double acc = 0.0;
  const float inv = 1.0f / (3.0f * (float)V);
  for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < V; v += stride) {
    __align__(16) bf16 row[NN_CH];
#pragma unroll
    for (int c = 0; c < NN_CH; c++) row[c] = __float2bfloat16_rn(0.f);
#pragma unroll
    for (int c = 0; c < 3; c++) {
      const float e = s * out[v * 4 + c] - tgt[v * 4 + c];
      acc += (double)e * e;
      row[c] = __float2bfloat16_rn(2.0f * e * s * inv);
    }
    reinterpret_cast<uint4 *>(g + v * NN_CH)[0] = reinterpret_cast<uint4 *>(row)[0];
    reinterpret_cast<uint4 *>(g + v * NN_CH)[1] = reinterpret_cast<uint4 *>(row)[1];
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += sh[w];
    atomicAdd(loss, t / (3.0 * (double)V));
  }
}

// Adam (Kingma & Ba 2015) on FP32 masters; writes the BF16 copy.  `live`
// masks the output channels a layer actually has (3 for the last layer).
__global__ void k_adam(float *__restrict__ w, const float *__restrict__ g, float *__restrict__ m,
                       float *__restrict__ v, bf16 *__restrict__ w16, int n, int stride_out, int live, float lr,
                       float b1, float b2, float eps, float c1, float c2) {
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
    const int o = (q / stride_out) % NN_CH;
    if (o >= live) {
      w[q] = 0.f;
      if (w16) w16[q] = __float2bfloat16_rn(0.f);
      continue;
    }
    const float gq = g[q];
    const float mq = b1 * m[q] + (1.f - b1) * gq, vq = b2 * v[q] + (1.f - b2) * gq * gq;
    m[q] = mq;
    v[q] = vq;
    const float wq = w[q] - lr * (mq / c1) / (sqrtf(vq / c2) + eps);
    w[q] = wq;
    if (w16) w16[q] = __float2bfloat16_rn(wq);
  }
}

__global__ void k_to_bf16(const float *__restrict__ a, bf16 *__restrict__ b, int n) {
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) b[q] = __float2bfloat16_rn(a[q]);
}

// Features per voxel from delta(x) (= grid_a / N^3) and Phi_N(x) (grid_b).
__global__ void k_features(const float *__restrict__ ga, const float *__restrict__ gb, int N, long long P,
                           float inv_n3, float phicrit, int screened, bf16 *__restrict__ X) {
  const long long V = (long long)N * N * N;
  long long stride = (long long)gridDim.x * blockDim.x;
  for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < V; v += stride) {
    const long long row = v / N;
    const int k = (int)(v - row * N);
    const long long g = row * P + k;
    const float d = ga[g] * inv_n3, ph = gb[g];
    float sc = 1.f;
    if (screened && ph < 0.f) sc = fminf(1.f, fabsf(phicrit / ph));
    __align__(16) bf16 rowv[NN_CH];
#pragma unroll
    for (int c = 0; c < NN_CH; c++) rowv[c] = __float2bfloat16_rn(0.f);
    rowv[0] = __float2bfloat16_rn(asinhf(d));
    rowv[1] = __float2bfloat16_rn(asinhf(ph * 1e5f));
    rowv[2] = __float2bfloat16_rn(sc);
    reinterpret_cast<uint4 *>(X + v * NN_CH)[0] = reinterpret_cast<uint4 *>(rowv)[0];
    reinterpret_cast<uint4 *>(X + v * NN_CH)[1] = reinterpret_cast<uint4 *>(rowv)[1];
  }
}

// Residual target on the coarse mesh: the fine force averaged over the
// 3 x 3 x 3 fine points around the coarse point (fine point r i), minus the
// coarse force.
__global__ void k_target(const float *__restrict__ ff, long long fg, int Nf, long long Pf, const float *__restrict__ fc,
                         long long cg, int N, long long P, int r, float *__restrict__ tgt) {
  const long long V = (long long)N * N * N;
  long long stride = (long long)gridDim.x * blockDim.x;
  const int h = r / 2;  // half-width of the averaging cube
  const float inv = 1.0f / (float)((2 * h + 1) * (2 * h + 1) * (2 * h + 1));
  for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < V; v += stride) {
    const int k = (int)(v % N), j = (int)((v / N) % N), i = (int)(v / ((long long)N * N));
    float s[3] = {0.f, 0.f, 0.f};
    for (int a = -h; a <= h; a++)
      for (int b = -h; b <= h; b++)
        for (int c = -h; c <= h; c++) {
          const int fi = (r * i + a + Nf) % Nf, fj = (r * j + b + Nf) % Nf, fk = (r * k + c + Nf) % Nf;
          const long long g = ((long long)fi * Nf + fj) * Pf + fk;
#pragma unroll
          for (int q = 0; q < 3; q++) s[q] += ff[q * fg + g];
        }
    const long long gc = ((long long)i * N + j) * P + k;
#pragma unroll
    for (int q = 0; q < 3; q++) tgt[v * 4 + q] = s[q] * inv - fc[q * cg + gc];
    tgt[v * 4 + 3] = 0.f;
  }
}

// Training-set compaction: 3 feature channels (bf16) and 3 target
// components (f32) per voxel.
__global__ void k_pack_sample(const bf16 *__restrict__ X, const float *__restrict__ t, long long V,
                              bf16 *__restrict__ dx, float *__restrict__ dt) {
  long long stride = (long long)gridDim.x * blockDim.x;
  for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < V; v += stride)
#pragma unroll
    for (int c = 0; c < 3; c++) {
      dx[v * 3 + c] = X[v * NN_CH + c];
      dt[v * 3 + c] = t[v * 4 + c];
    }
}
__global__ void k_unpack_sample(const bf16 *__restrict__ dx, const float *__restrict__ dt, long long V,
                                bf16 *__restrict__ X, float *__restrict__ t) {
  long long stride = (long long)gridDim.x * blockDim.x;
  for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < V; v += stride) {
    __align__(16) bf16 rowv[NN_CH];
#pragma unroll
    for (int c = 0; c < NN_CH; c++) rowv[c] = __float2bfloat16_rn(0.f);
#pragma unroll
    for (int c = 0; c < 3; c++) {
      rowv[c] = dx[v * 3 + c];
      t[v * 4 + c] = dt[v * 3 + c];
    }
    t[v * 4 + 3] = 0.f;
    reinterpret_cast<uint4 *>(X + v * NN_CH)[0] = reinterpret_cast<uint4 *>(rowv)[0];
    reinterpret_cast<uint4 *>(X + v * NN_CH)[1] = reinterpret_cast<uint4 *>(rowv)[1];
  }
}

}  // namespace

// --------------------------------------------------------------- host side
#define NN_RET(x)                  \
  do {                             \
    int rc_ = (x);                 \
    if (rc_ != MGP_OK) return rc_; \
  } while (0)

static int conv_fwd(mgp_closure *cl, const bf16 *X, const bf16 *W, const float *bias, int mode, bf16 *Y16, float *Y32,
                    float *frc, long long gstride, long long P, float scale) {
  const int N = cl->N, nseg = (N + NN_SEG - 1) / NN_SEG;
  const long long blocks = (long long)N * N * nseg;
  k_conv_fwd<<<(unsigned)blocks, kThreadsConv, 0, cl->stream>>>(X, W, bias, N, mode, Y16, Y32, frc, gstride, P, scale);
  MGP_CHECK_LAUNCH();
  g_kernel_launches++;
  return MGP_OK;
}

static int conv_wgrad(mgp_closure *cl, const bf16 *X, const bf16 *dY, float *dW, float *db) {
  int sms = 152;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, cl->device);
  const int nseg = (cl->N + NN_SEG - 1) / NN_SEG;
  long long units = (long long)cl->N * cl->N * nseg, blocks = (long long)sms * 4;
  if (blocks > units) blocks = units;
  k_conv_wgrad<<<(unsigned)blocks, kThreadsWg, 0, cl->stream>>>(X, dY, cl->N, dW, db);
  MGP_CHECK_LAUNCH();
  g_kernel_launches++;
  return MGP_OK;
}

static int closure_forward(mgp_closure *cl) {
  for (int l = 0; l < NN_LAYERS - 1; l++)
    NN_RET(conv_fwd(cl, cl->act[l], cl->w16[l], cl->b32[l], 0, cl->act[l + 1], NULL, NULL, 0, 0, 0.f));
  return conv_fwd(cl, cl->act[NN_LAYERS - 1], cl->w16[NN_LAYERS - 1], cl->b32[NN_LAYERS - 1], 2, NULL, cl->out, NULL,
                  0, 0, 0.f);
}

// Loss and all gradients for the current features/target.
static int closure_backward(mgp_closure *cl) {
  const long long V = cl->V;
  MGP_CUDA(cudaMemsetAsync(cl->loss, 0, sizeof(double), cl->stream));
  k_loss_grad<<<mgp_blocks_for(V, 4), 256, 0, cl->stream>>>(cl->out, cl->target, V, cl->out_scale, cl->g0, cl->loss);
  MGP_CHECK_LAUNCH();
  g_kernel_launches++;
  bf16 *g = cl->g0, *gn = cl->g1;
  for (int l = NN_LAYERS - 1; l >= 0; l--) {
    MGP_CUDA(cudaMemsetAsync(cl->gw[l], 0, sizeof(float) * NN_WSIZE, cl->stream));
    MGP_CUDA(cudaMemsetAsync(cl->gb[l], 0, sizeof(float) * NN_CH, cl->stream));
    NN_RET(conv_wgrad(cl, cl->act[l], g, cl->gw[l], cl->gb[l]));
    if (l == 0) break;
    k_mirror_transpose<<<(NN_WSIZE + 255) / 256, 256, 0, cl->stream>>>(cl->w16[l], cl->wt16);
    MGP_CHECK_LAUNCH();
    g_kernel_launches++;
    NN_RET(conv_fwd(cl, g, cl->wt16, NULL, 1, gn, NULL, NULL, 0, 0, 0.f));
    k_relu_grad<<<mgp_blocks_for(V * NN_CH, 4), 256, 0, cl->stream>>>(gn, cl->act[l], V * NN_CH);
    MGP_CHECK_LAUNCH();
    g_kernel_launches++;
    bf16 *t = g;
    g = gn;
    gn = t;
  }
  return MGP_OK;
}

static int sync_weights16(mgp_closure *cl) {
  for (int l = 0; l < NN_LAYERS; l++) {
    k_to_bf16<<<(NN_WSIZE + 255) / 256, 256, 0, cl->stream>>>(cl->w32[l], cl->w16[l], NN_WSIZE);
    MGP_CHECK_LAUNCH();
  }
  return MGP_OK;
}

extern "C" int mgp_closure_destroy(mgp_closure *cl) {
  if (!cl) return MGP_OK;
  cudaSetDevice(cl->device);
  if (cl->stream) cudaStreamSynchronize(cl->stream);
  for (int l = 0; l < NN_LAYERS; l++) {
    void *b[] = {cl->w32[l], cl->b32[l], cl->gw[l], cl->gb[l], cl->mw[l], cl->vw[l], cl->mb[l], cl->vb[l], cl->w16[l],
                 cl->act[l]};
    for (size_t q = 0; q < sizeof(b) / sizeof(b[0]); q++)
      if (b[q]) cudaFree(b[q]);
  }
  void *b[] = {cl->wt16, cl->out, cl->target, cl->g0, cl->g1, cl->loss, cl->grid_a, cl->grid_b, cl->ds_x, cl->ds_t};
  for (size_t q = 0; q < sizeof(b) / sizeof(b[0]); q++)
    if (b[q]) cudaFree(b[q]);
  if (cl->own_stream && cl->stream) cudaStreamDestroy(cl->stream);
  free(cl);
  return MGP_OK;
}

// Deterministic He-normal initialisation (Box-Muller on a 64-bit LCG).
static void init_weights(std::vector<float> &w, int fan_in, int live, uint64_t &st) {
  const double sd = sqrt(2.0 / (double)fan_in);
  for (size_t q = 0; q < w.size(); q++) {
    st = st * 6364136223846793005ULL + 1442695040888963407ULL;
    double u1 = ((st >> 11) + 1.0) / 9007199254740993.0;
    st = st * 6364136223846793005ULL + 1442695040888963407ULL;
    double u2 = (st >> 11) / 9007199254740992.0;
    const int o = (int)((q / NN_CH) % NN_CH);
    w[q] = o < live ? (float)(sd * sqrt(-2.0 * log(u1)) * cos(2.0 * M_PI * u2)) : 0.f;
  }
}

extern "C" int mgp_closure_create(int Nmesh, unsigned seed, int device, mgp_closure **out) {
  if (!out) return mgp_set_error(MGP_EINVAL, "null argument");
  *out = NULL;
  if (Nmesh < 16 || Nmesh % 16) return mgp_set_error(MGP_EINVAL, "closure needs Nmesh a multiple of 16 (%d)", Nmesh);
  MGP_CUDA(cudaSetDevice(device));
  mgp_closure *cl = (mgp_closure *)calloc(1, sizeof(mgp_closure));
  cl->N = Nmesh;
  cl->V = (long long)Nmesh * Nmesh * Nmesh;
  cl->device = device;
  cl->P = 2LL * (Nmesh / 2 + 1);
  cl->out_scale = 1.0f;
#define CL_TRY(x)                        \
  do {                                   \
    cudaError_t e_ = (x);                \
    if (e_ != cudaSuccess) {             \
      mgp_closure_destroy(cl);           \
      return mgp_set_error(MGP_ECUDA, "closure: %s", cudaGetErrorString(e_)); \
    }                                    \
  } while (0)
  CL_TRY(cudaStreamCreateWithFlags(&cl->stream, cudaStreamNonBlocking));
  cl->own_stream = 1;
  uint64_t st = 0x9E3779B97F4A7C15ULL ^ seed;
  for (int l = 0; l < NN_LAYERS; l++) {
    float **f[] = {&cl->w32[l], &cl->gw[l], &cl->mw[l], &cl->vw[l]};
    for (int q = 0; q < 4; q++) {
      CL_TRY(cudaMalloc(f[q], sizeof(float) * NN_WSIZE));
      CL_TRY(cudaMemset(*f[q], 0, sizeof(float) * NN_WSIZE));
    }
    float **g[] = {&cl->b32[l], &cl->gb[l], &cl->mb[l], &cl->vb[l]};
    for (int q = 0; q < 4; q++) {
      CL_TRY(cudaMalloc(g[q], sizeof(float) * NN_CH));
      CL_TRY(cudaMemset(*g[q], 0, sizeof(float) * NN_CH));
    }
    CL_TRY(cudaMalloc(&cl->w16[l], sizeof(bf16) * NN_WSIZE));
    CL_TRY(cudaMalloc(&cl->act[l], sizeof(bf16) * NN_CH * cl->V));
    CL_TRY(cudaMemset(cl->act[l], 0, sizeof(bf16) * NN_CH * cl->V));
    std::vector<float> w(NN_WSIZE);
    // fan-in: 27 taps x (3 live inputs for the first layer, 16 otherwise)
    init_weights(w, NN_TAPS * (l == 0 ? 3 : NN_CH), l == NN_LAYERS - 1 ? 3 : NN_CH, st);
    if (l == NN_LAYERS - 1)
      for (auto &x : w) x *= 0.1f;  // start near the plain PM force
    CL_TRY(cudaMemcpy(cl->w32[l], w.data(), sizeof(float) * NN_WSIZE, cudaMemcpyHostToDevice));
  }
  CL_TRY(cudaMalloc(&cl->wt16, sizeof(bf16) * NN_WSIZE));
  CL_TRY(cudaMalloc(&cl->out, sizeof(float) * 4 * cl->V));
  CL_TRY(cudaMalloc(&cl->target, sizeof(float) * 4 * cl->V));
  CL_TRY(cudaMemset(cl->target, 0, sizeof(float) * 4 * cl->V));
  CL_TRY(cudaMalloc(&cl->g0, sizeof(bf16) * NN_CH * cl->V));
  CL_TRY(cudaMalloc(&cl->g1, sizeof(bf16) * NN_CH * cl->V));
  CL_TRY(cudaMalloc(&cl->loss, sizeof(double)));
#undef CL_TRY
  int rc = sync_weights16(cl);
  if (rc == MGP_OK) rc = cudaStreamSynchronize(cl->stream) == cudaSuccess ? MGP_OK : MGP_ECUDA;
  if (rc) {
    mgp_closure_destroy(cl);
    return mgp_set_error(rc, "closure initialisation failed");
  }
  *out = cl;
  return MGP_OK;
}

// Weights as FP32 host arrays: w [4][27][16][16], b [4][16]; scale = out_scale.
extern "C" int mgp_closure_get_weights(mgp_closure *cl, float *w, float *b, float *scale) {
  if (!cl) return mgp_set_error(MGP_EINVAL, "null closure");
  MGP_CUDA(cudaStreamSynchronize(cl->stream));
  for (int l = 0; l < NN_LAYERS; l++) {
    if (w) MGP_CUDA(cudaMemcpy(w + l * NN_WSIZE, cl->w32[l], sizeof(float) * NN_WSIZE, cudaMemcpyDeviceToHost));
    if (b) MGP_CUDA(cudaMemcpy(b + l * NN_CH, cl->b32[l], sizeof(float) * NN_CH, cudaMemcpyDeviceToHost));
  }
  if (scale) *scale = cl->out_scale;
  return MGP_OK;
}

extern "C" int mgp_closure_set_weights(mgp_closure *cl, const float *w, const float *b, float scale) {
  if (!cl) return mgp_set_error(MGP_EINVAL, "null closure");
  MGP_CUDA(cudaStreamSynchronize(cl->stream));
  for (int l = 0; l < NN_LAYERS; l++) {
    if (w) MGP_CUDA(cudaMemcpy(cl->w32[l], w + l * NN_WSIZE, sizeof(float) * NN_WSIZE, cudaMemcpyHostToDevice));
    if (b) MGP_CUDA(cudaMemcpy(cl->b32[l], b + l * NN_CH, sizeof(float) * NN_CH, cudaMemcpyHostToDevice));
  }
  if (scale > 0) cl->out_scale = scale;
  NN_RET(sync_weights16(cl));
  MGP_CUDA(cudaStreamSynchronize(cl->stream));
  return MGP_OK;
}

// Host features [V][3] / targets [V][3] (FP32) into the working buffers.
extern "C" int mgp_closure_set_sample(mgp_closure *cl, const float *x, const float *t) {
  if (!cl) return mgp_set_error(MGP_EINVAL, "null closure");
  const long long V = cl->V;
  if (x) {
    std::vector<bf16> h((size_t)V * NN_CH);
    for (long long v = 0; v < V; v++)
      for (int c = 0; c < NN_CH; c++) h[v * NN_CH + c] = __float2bfloat16_rn(c < 3 ? x[v * 3 + c] : 0.f);
    MGP_CUDA(cudaMemcpy(cl->act[0], h.data(), sizeof(bf16) * h.size(), cudaMemcpyHostToDevice));
  }
  if (t) {
    std::vector<float> h((size_t)V * 4, 0.f);
    for (long long v = 0; v < V; v++)
      for (int c = 0; c < 3; c++) h[v * 4 + c] = t[v * 3 + c];
    MGP_CUDA(cudaMemcpy(cl->target, h.data(), sizeof(float) * h.size(), cudaMemcpyHostToDevice));
  }
  return MGP_OK;
}

// Forward pass on the working features; out [V][3] host (may be NULL).
extern "C" int mgp_closure_forward(mgp_closure *cl, float *out) {
  if (!cl) return mgp_set_error(MGP_EINVAL, "null closure");
  MGP_CUDA(cudaSetDevice(cl->device));
  NN_RET(closure_forward(cl));
  MGP_CUDA(cudaStreamSynchronize(cl->stream));
  if (out) {
    std::vector<float> h((size_t)cl->V * 4);
    MGP_CUDA(cudaMemcpy(h.data(), cl->out, sizeof(float) * h.size(), cudaMemcpyDeviceToHost));
    for (long long v = 0; v < cl->V; v++)
      for (int c = 0; c < 3; c++) out[v * 3 + c] = h[v * 4 + c];
  }
  return MGP_OK;
}

// Loss and gradients (no update); gw [4][27][16][16], gb [4][16] host.
extern "C" int mgp_closure_gradients(mgp_closure *cl, double *loss, float *gw, float *gb) {
  if (!cl) return mgp_set_error(MGP_EINVAL, "null closure");
  MGP_CUDA(cudaSetDevice(cl->device));
  NN_RET(closure_forward(cl));
  NN_RET(closure_backward(cl));
  MGP_CUDA(cudaStreamSynchronize(cl->stream));
  if (loss) MGP_CUDA(cudaMemcpy(loss, cl->loss, sizeof(double), cudaMemcpyDeviceToHost));
  for (int l = 0; l < NN_LAYERS; l++) {
    if (gw) MGP_CUDA(cudaMemcpy(gw + l * NN_WSIZE, cl->gw[l], sizeof(float) * NN_WSIZE, cudaMemcpyDeviceToHost));
    if (gb) MGP_CUDA(cudaMemcpy(gb + l * NN_CH, cl->gb[l], sizeof(float) * NN_CH, cudaMemcpyDeviceToHost));
  }
  return MGP_OK;
}

// One Adam step on the working sample; returns the loss before the update.
extern "C" int mgp_closure_train_step(mgp_closure *cl, float lr, double *loss) {
  if (!cl) return mgp_set_error(MGP_EINVAL, "null closure");
  MGP_CUDA(cudaSetDevice(cl->device));
  NN_RET(closure_forward(cl));
  NN_RET(closure_backward(cl));
  cl->adam_t++;
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  const float c1 = 1.f - powf(b1, (float)cl->adam_t), c2 = 1.f - powf(b2, (float)cl->adam_t);
  for (int l = 0; l < NN_LAYERS; l++) {
    const int live = l == NN_LAYERS - 1 ? 3 : NN_CH;
    k_adam<<<(NN_WSIZE + 255) / 256, 256, 0, cl->stream>>>(cl->w32[l], cl->gw[l], cl->mw[l], cl->vw[l], cl->w16[l],
                                                            NN_WSIZE, NN_CH, live, lr, b1, b2, eps, c1, c2);
    MGP_CHECK_LAUNCH();
    k_adam<<<1, NN_CH, 0, cl->stream>>>(cl->b32[l], cl->gb[l], cl->mb[l], cl->vb[l], NULL, NN_CH, 1, live, lr, b1, b2,
                                        eps, c1, c2);
    MGP_CHECK_LAUNCH();
  }
  if (loss) {
    MGP_CUDA(cudaMemcpyAsync(loss, cl->loss, sizeof(double), cudaMemcpyDeviceToHost, cl->stream));
    MGP_CUDA(cudaStreamSynchronize(cl->stream));
  }
  return MGP_OK;
}

// ------------------------------------------------ the closure on a PM mesh
// Features of a context's current density: delta(x) and Phi_N(x) from its
// delta(k) (two C2R on the closure's scratch grids, the context's plan).
static int closure_features(mgp_closure *cl, mgp_ctx *c, double A) {
  const int N = c->g.N;
  const long long gf = c->g.nreal;
  if (!cl->grid_a) {
    MGP_CUDA(cudaMalloc(&cl->grid_a, sizeof(float) * gf));
    MGP_CUDA(cudaMalloc(&cl->grid_b, sizeof(float) * gf));
  }
  MGP_CUFFT(cufftSetStream(c->plan_c2r_1, cl->stream));
  MGP_CUDA(cudaMemcpyAsync(cl->grid_a, c->dk, sizeof(float) * gf, cudaMemcpyDeviceToDevice, cl->stream));
  const mgp_params *p = &c->p;
  const double norm = 1.0 / pow((double)N, 3) * 1.5 * p->Omega / A * pow(p->Box / 2997.92458 / (2.0 * M_PI), 2);
  NN_RET(mgp_launch_div_laplacian(c->dk, cl->grid_b, N, (float)norm, cl->stream));
  cufftResult r1 = cufftExecC2R(c->plan_c2r_1, (cufftComplex *)cl->grid_a, (cufftReal *)cl->grid_a);
  cufftResult r2 = cufftExecC2R(c->plan_c2r_1, (cufftComplex *)cl->grid_b, (cufftReal *)cl->grid_b);
  cufftSetStream(c->plan_c2r_1, c->stream);
  if (r1 != CUFFT_SUCCESS || r2 != CUFFT_SUCCESS) return mgp_set_error(MGP_ECUFFT, "closure feature transforms");
  const int screened = p->modified_gravity_active && p->include_screening &&
                       (p->model == MGP_MODEL_FOFR || p->model == MGP_MODEL_MBETA);
  const float phicrit = screened ? (float)mgp_phicrit(&c->cosmo, A) : 0.f;
  k_features<<<mgp_blocks_for(cl->V, 4), 256, 0, cl->stream>>>(cl->grid_a, cl->grid_b, N, c->g.P,
                                                               (float)(1.0 / pow((double)N, 3)), phicrit, screened,
                                                               cl->act[0]);
  MGP_CHECK_LAUNCH();
  g_kernel_launches++;
  return MGP_OK;
}

static int check_ctx(mgp_closure *cl, mgp_ctx *c) {
  if (!cl || !c) return mgp_set_error(MGP_EINVAL, "null closure or context");
  if (c->nbox != 1) return mgp_set_error(MGP_EINVAL, "the closure works on single-box contexts");
  if (c->g.N != cl->N) return mgp_set_error(MGP_EINVAL, "closure mesh %d vs context mesh %d", cl->N, c->g.N);
  if (!c->have_forces) return mgp_set_error(MGP_ESTATE, "context has no forces: call mgp_get_displacements first");
  return MGP_OK;
}

// Training input from a coarse context after mgp_get_displacements(A).
extern "C" int mgp_closure_features(mgp_closure *cl, mgp_ctx *c, double A) {
  NN_RET(check_ctx(cl, c));
  MGP_CUDA(cudaSetDevice(cl->device));
  MGP_CUDA(cudaStreamSynchronize(c->stream));
  NN_RET(closure_features(cl, c, A));
  MGP_CUDA(cudaStreamSynchronize(cl->stream));
  return MGP_OK;
}

__global__ void k_sumsq(const float *__restrict__ t, long long V, double *__restrict__ out) {
  __shared__ double sh[8];
  double acc = 0.0;
  for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < V; v += (long long)gridDim.x * blockDim.x)
    for (int c = 0; c < 3; c++) acc += (double)t[v * 4 + c] * t[v * 4 + c];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) s += sh[w];
    atomicAdd(out, s);
  }
}

// Training target: the force of a fine context (Nmesh = r N, same particles
// and scale factor) averaged onto the coarse mesh, minus the coarse force;
// *rms (optional) receives its rms over voxels and components.
extern "C" int mgp_closure_target(mgp_closure *cl, mgp_ctx *fine, mgp_ctx *coarse, double *rms) {
  NN_RET(check_ctx(cl, coarse));
  if (!fine || fine->nbox != 1 || !fine->have_forces) return mgp_set_error(MGP_ESTATE, "fine context has no forces");
  const int Nf = fine->g.N, N = coarse->g.N;
  if (Nf % N) return mgp_set_error(MGP_EINVAL, "fine mesh %d is not a multiple of %d", Nf, N);
  MGP_CUDA(cudaSetDevice(cl->device));
  MGP_CUDA(cudaStreamSynchronize(fine->stream));
  MGP_CUDA(cudaStreamSynchronize(coarse->stream));
  k_target<<<mgp_blocks_for(cl->V, 4), 256, 0, cl->stream>>>(fine->frc, fine->g.nreal, Nf, fine->g.P, coarse->frc,
                                                             coarse->g.nreal, N, coarse->g.P, Nf / N, cl->target);
  MGP_CHECK_LAUNCH();
  g_kernel_launches++;
  if (rms) {
    MGP_CUDA(cudaMemsetAsync(cl->loss, 0, sizeof(double), cl->stream));
    k_sumsq<<<mgp_blocks_for(cl->V, 4), 256, 0, cl->stream>>>(cl->target, cl->V, cl->loss);
    MGP_CHECK_LAUNCH();
    double s = 0.0;
    MGP_CUDA(cudaMemcpyAsync(&s, cl->loss, sizeof(double), cudaMemcpyDeviceToHost, cl->stream));
    MGP_CUDA(cudaStreamSynchronize(cl->stream));
    *rms = sqrt(s / (3.0 * (double)cl->V));
  }
  MGP_CUDA(cudaStreamSynchronize(cl->stream));
  return MGP_OK;
}

// Training set on the device: `n` slots of (3 feature channels, 3 target
// components) per voxel.
extern "C" int mgp_closure_reserve(mgp_closure *cl, int n) {
  if (!cl || n < 0) return mgp_set_error(MGP_EINVAL, "bad closure reserve");
  MGP_CUDA(cudaSetDevice(cl->device));
  MGP_CUDA(cudaStreamSynchronize(cl->stream));
  if (cl->ds_x) cudaFree(cl->ds_x);
  if (cl->ds_t) cudaFree(cl->ds_t);
  cl->ds_x = NULL;
  cl->ds_t = NULL;
  cl->cap_samples = cl->nsamples = 0;
  if (n == 0) return MGP_OK;
  MGP_CUDA(cudaMalloc(&cl->ds_x, sizeof(bf16) * 3 * cl->V * n));
  MGP_CUDA(cudaMalloc(&cl->ds_t, sizeof(float) * 3 * cl->V * n));
  cl->cap_samples = n;
  return MGP_OK;
}

extern "C" int mgp_closure_store(mgp_closure *cl, int slot) {
  if (!cl || slot < 0 || slot >= cl->cap_samples) return mgp_set_error(MGP_EINVAL, "bad closure slot %d", slot);
  k_pack_sample<<<mgp_blocks_for(cl->V, 4), 256, 0, cl->stream>>>(cl->act[0], cl->target, cl->V,
                                                                  cl->ds_x + (size_t)slot * 3 * cl->V,
                                                                  cl->ds_t + (size_t)slot * 3 * cl->V);
  MGP_CHECK_LAUNCH();
  if (slot >= cl->nsamples) cl->nsamples = slot + 1;
  MGP_CUDA(cudaStreamSynchronize(cl->stream));
  return MGP_OK;
}

extern "C" int mgp_closure_load(mgp_closure *cl, int slot) {
  if (!cl || slot < 0 || slot >= cl->nsamples) return mgp_set_error(MGP_EINVAL, "bad closure slot %d", slot);
  k_unpack_sample<<<mgp_blocks_for(cl->V, 4), 256, 0, cl->stream>>>(cl->ds_x + (size_t)slot * 3 * cl->V,
                                                                    cl->ds_t + (size_t)slot * 3 * cl->V, cl->V,
                                                                    cl->act[0], cl->target);
  MGP_CHECK_LAUNCH();
  return MGP_OK;
}

// Inference inside a PM step (called by mgp_get_displacements after the
// force grids): features, three hidden layers and the last layer added to the
// force grids, on the context's stream.
int mgp_closure_apply(mgp_closure *cl, mgp_ctx *c, double A) {
  cudaStream_t keep = cl->stream;
  cl->stream = c->stream;
  int rc = closure_features(cl, c, A);
  for (int l = 0; l < NN_LAYERS - 1 && rc == MGP_OK; l++)
    rc = conv_fwd(cl, cl->act[l], cl->w16[l], cl->b32[l], 0, cl->act[l + 1], NULL, NULL, 0, 0, 0.f);
  if (rc == MGP_OK)
    rc = conv_fwd(cl, cl->act[NN_LAYERS - 1], cl->w16[NN_LAYERS - 1], cl->b32[NN_LAYERS - 1], 3, NULL, NULL, c->frc,
                  c->g.nreal, c->g.P, cl->out_scale);
  cl->stream = keep;
  return rc;
}

// Attach (cl != NULL) or detach a closure: every later mgp_get_displacements
// of the context adds the closure's residual force.
extern "C" int mgp_set_closure(mgp_ctx *c, mgp_closure *cl) {
  if (!c) return mgp_set_error(MGP_EINVAL, "null context");
  if (cl && (c->nbox != 1 || c->g.N != cl->N))
    return mgp_set_error(MGP_EINVAL, "closure mesh %d does not fit the context", cl ? cl->N : 0);
  if (cl && c->sd) return mgp_set_error(MGP_EINVAL, "the closure runs with scale-independent growth");
  c->closure = cl;
  return MGP_OK;
}

// The working sample back on the host: features [V][3] and target [V][3].
extern "C" int mgp_closure_get_sample(mgp_closure *cl, float *x, float *t) {
  if (!cl) return mgp_set_error(MGP_EINVAL, "null closure");
  MGP_CUDA(cudaStreamSynchronize(cl->stream));
  const long long V = cl->V;
  if (x) {
    std::vector<bf16> h((size_t)V * NN_CH);
    MGP_CUDA(cudaMemcpy(h.data(), cl->act[0], sizeof(bf16) * h.size(), cudaMemcpyDeviceToHost));
    for (long long v = 0; v < V; v++)
      for (int c = 0; c < 3; c++) x[v * 3 + c] = __bfloat162float(h[v * NN_CH + c]);
  }
  if (t) {
    std::vector<float> h((size_t)V * 4);
    MGP_CUDA(cudaMemcpy(h.data(), cl->target, sizeof(float) * h.size(), cudaMemcpyDeviceToHost));
    for (long long v = 0; v < V; v++)
      for (int c = 0; c < 3; c++) t[v * 3 + c] = h[v * 4 + c];
  }
  return MGP_OK;
}
