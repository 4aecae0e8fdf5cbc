// Learned force closure: a small 3D CNN on the PM mesh that predicts the
// residual between the force of a finer mesh and the mesh force, trained on
// the GPU by the kernels of this file (no counterpart in the reference).
//
// Network: four periodic 3x3x3 convolutions, 16 channels between layers,
// ReLU after the first three, the last layer linear with 3 outputs (the
// residual force components).  Inputs per cell (padded to 16 channels):
// asinh(delta), Phi_N / 1e-5 (linear: the resolution correction is to
// first order a linear filter of the potential) and the screening factor
// min(1, |phi_crit / Phi_N|) for Phi_N < 0 (1 otherwise, and 1 for models
// without potential screening).  Activations and weights are BF16, every
// accumulation is FP32 on the tensor cores (mma.sync m16n8k16 bf16).
//
// Layout: activations channel-last [V][16] bf16 with voxel v = (i N + j) N + k
// (k fastest, as the mesh rows); weights [27 taps][16 out][16 in], tap =
// 9 (di+1) + 3 (dj+1) + (dk+1) for offsets d in {-1, 0, 1}.
//
// Convolution as implicit GEMM (k_conv_fwd): persistent blocks keep all
// weights in shared memory and walk tiles of 2 x 4 output rows (i, j) by 64
// voxels; a tile stages the 4 x 6 input rows around it once (cp.async), and
// warp w computes one output row as 4 groups of 16 voxels, each tap one
// 16x16x16 product (two m16n8k16 MMAs) whose A fragment is the staged row
// shifted by dk (ldmatrix).  With 16 channels the product per tap is N = 16
// wide: a tcgen05 version (M = 128 voxels, N = 16, K = 16 per tap, TMEM
// accumulators) measured 1.5x slower per layer on the same 192^3 input, its
// MMAs bound by per-instruction operand fetch rather than the datapath, so
// the register-blocked mma.sync kernel is the one used.  The data gradient is
// the same convolution with the weights mirrored (tap -> 26 - tap) and
// transposed (in <-> out); the weight gradient is, per tap, dY^T X over all
// voxels, accumulated by persistent blocks in registers and reduced with one
// FP32 atomic per weight per block.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <vector>

#include "mgp_device.cuh"
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
  // particle-level target (pmode 1): cell coordinates on this mesh and
  // r_p = F_fine(x_p) - F_coarse(x_p), SoA [3][np]; cur_* point at the
  // working sample (own buffers or a stored slot)
  int pmode;
  long long np;                            // particles of the working sample
  float pscale;                            // output scale of the working particle sample
  int pnorm;                               // 1: its loss is relative to pscale^2 (samples from contexts)
  long long own_np;                        // capacity of pc / pt
  float *pc, *pt;
  const float *cur_pc, *cur_pt;
  // high-passed network output and its gradient (particle loss and the
  // in-step path): three padded real grids each, [3][N][N][P]
  float *ugrid, *dgrid;
  cufftHandle plan_r2c, plan_c2r;          // in-place N^3 transforms of one grid
  int have_plans;
  float hp_lambda;                         // high-pass cutoff wavelength in cells (0: only the mean removed)
  float *fscr;                             // band-limited fine force, 3 fine grids (lazy)
  float *wg_partial;                       // weight-gradient partial sums per block (lazy)
  int wg_blocks;
  long long fscr_floats;
  // stored training samples: features (3 bf16) per voxel and either grid
  // targets (3 f32 per voxel, ds_np = 0) or particle samples (ds_np > 0)
  int nsamples, cap_samples;
  long long ds_np;
  bf16 *ds_x;
  float *ds_t, *ds_pc, *ds_pt;
  float *ds_s;                             // host: output scale per stored particle sample
  // residual scale vs scale factor for the in-step path (log-log table; n = 0: out_scale)
  int scale_n;
  double *scale_a, *scale_s;
};

namespace {


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

// Forward convolution, persistent: a CTA keeps all weights in shared memory
// and walks tiles of CT_I x CT_J output rows (i, j) by CT_SEG voxels (k).
// For a tile it stages the (CT_I+2) x (CT_J+2) input rows around it, each
// with one halo voxel on either side (cp.async), so a staged row serves up
// to 9 output rows; warp w computes output row (i0 + w / CT_J, j0 + w % CT_J)
// as 4 groups of 16 voxels, reusing each tap's B fragment for the 4 groups.
// Shared-memory layout of a [voxel][16] bf16 row: the two 16-byte halves of
// voxel q are swapped when bit 2 of q is set, so the 8 row addresses of any
// ldmatrix (8 consecutive voxels or 8 consecutive output channels) fall in 8
// distinct 16-byte bank groups.
// mode 0: bf16 out, bias + ReLU; 1: bf16 out, no bias, times relu'(gate)
// (data gradient through the previous layer's ReLU, gate = its output); 2: f32
// out [V][4] (channels 0-3), bias; 3: out + bias into three padded real
// grids (channels 0-2; grid c at frc + c gstride, rows of P floats).
constexpr int CT_I = 2, CT_J = 4, CT_SEG = 64;
constexpr int CT_ROWS = (CT_I + 2) * (CT_J + 2);  // staged rows
constexpr int CT_Q = CT_SEG + 2;                  // staged voxels per row
constexpr int kThreadsConv = 32 * CT_I * CT_J;    // one warp per output row
constexpr size_t kConvSmem = sizeof(bf16) * (NN_WSIZE + (size_t)CT_ROWS * CT_Q * NN_CH);

__device__ __forceinline__ int swz_half(int q, int h) { return h ^ ((q >> 2) & 1); }
__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(smem_u32(smem)), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;\n" ::: "memory");
}

__global__ void __launch_bounds__(kThreadsConv, 3) k_conv_fwd(const bf16 *__restrict__ X, const bf16 *__restrict__ W,
                                                              const float *__restrict__ bias,
                                                              const bf16 *__restrict__ gate, int N, int mode,
                                                              bf16 *__restrict__ Y16, float *__restrict__ Y32,
                                                              float *__restrict__ frc, long long gstride, long long P,
                                                              float scale) {
  extern __shared__ __align__(16) unsigned char conv_smem[];
  bf16(*ws)[NN_CH] = reinterpret_cast<bf16(*)[NN_CH]>(conv_smem);  // [tap * 16 + out][16 in]
  bf16(*xs)[CT_Q][NN_CH] = reinterpret_cast<bf16(*)[CT_Q][NN_CH]>(conv_smem + sizeof(bf16) * NN_WSIZE);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  for (int c = tid; c < NN_WSIZE / 8; c += kThreadsConv) {
    const int row = c >> 1, h = c & 1;  // row = tap * 16 + out
    cp_async16(&ws[row][8 * swz_half(row & 15, h)], W + (size_t)c * 8);
  }
  const int nseg = (N + CT_SEG - 1) / CT_SEG, tiles_j = N / CT_J;
  const long long ntiles = (long long)(N / CT_I) * tiles_j * nseg;
  const int wi = warp / CT_J, wj = warp % CT_J;
  // ldmatrix lane roles: A (16 voxels x 16 ch), B (16 out x 16 in)
  const int a_vox = (lane & 7) + 8 * ((lane >> 3) & 1), a_half = lane >> 4;
  const int b_out = (lane & 7) + 8 * (lane >> 4), b_half = (lane >> 3) & 1;
  const int vr = lane >> 2, cc = 2 * (lane & 3);
  for (long long t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int seg = (int)(t % nseg);
    const long long rest = t / nseg;
    const int i0 = (int)(rest / tiles_j) * CT_I, j0 = (int)(rest % tiles_j) * CT_J, k0 = seg * CT_SEG;
    const int qmax = min(CT_SEG + 1, N - k0 + 1);  // staged voxels past qmax are zero
    __syncthreads();  // the previous tile's reads of xs are done
    for (int c = tid; c < CT_ROWS * CT_Q * 2; c += kThreadsConv) {
      const int r = c / (CT_Q * 2), rem = c - r * (CT_Q * 2), q = rem >> 1, h = rem & 1;
      bf16 *dst = &xs[r][q][8 * swz_half(q, h)];
      if (q > qmax) {
        *reinterpret_cast<uint4 *>(dst) = make_uint4(0, 0, 0, 0);
        continue;
      }
      int ii = i0 + r / (CT_J + 2) - 1, jj = j0 + r % (CT_J + 2) - 1, kk = k0 - 1 + q;
      ii += ii < 0 ? N : 0;
      ii -= ii >= N ? N : 0;
      jj += jj < 0 ? N : 0;
      jj -= jj >= N ? N : 0;
      kk += kk < 0 ? N : 0;
      kk -= kk >= N ? N : 0;
      cp_async16(dst, X + (((long long)ii * N + jj) * N + kk) * NN_CH + 8 * h);
    }
    cp_async_wait_all();
    __syncthreads();
    const int ng = min(4, (N - k0) / 16);  // valid 16-voxel groups (N is a multiple of 16)
    float acc[4][2][4];
#pragma unroll
    for (int g = 0; g < 4; g++)
#pragma unroll
      for (int n = 0; n < 2; n++)
#pragma unroll
        for (int q = 0; q < 4; q++) acc[g][n][q] = 0.f;
#pragma unroll 3
    for (int tap = 0; tap < NN_TAPS; tap++) {
      const int di = tap / 9, dj = (tap / 3) % 3, dk = tap % 3;
      const int r = (wi + di) * (CT_J + 2) + (wj + dj);
      uint32_t b0, b1, b2, b3;
      ldsm_x4(smem_u32(&ws[tap * NN_CH + b_out][8 * swz_half(b_out, b_half)]), b0, b1, b2, b3);
#pragma unroll
      for (int g = 0; g < 4; g++) {
        if (g < ng) {
          const int q = 16 * g + a_vox + dk;
          uint32_t a0, a1, a2, a3;
          ldsm_x4(smem_u32(&xs[r][q][8 * swz_half(q, a_half)]), a0, a1, a2, a3);
          mma16816(acc[g][0], a0, a1, a2, a3, b0, b1);
          mma16816(acc[g][1], a0, a1, a2, a3, b2, b3);
        }
      }
    }
    // fragment: rows (voxels) lane/4 and lane/4 + 8, columns 2 (lane%4) + {0,1}
    const int i = i0 + wi, j = j0 + wj;
#pragma unroll
    for (int g = 0; g < 4; g++) {
      if (g >= ng) continue;
      const int kw = k0 + 16 * g;
      const long long vb = ((long long)i * N + j) * N + kw;
#pragma unroll
      for (int h = 0; h < 2; h++) {
        const long long v = vb + vr + 8 * h;
        float o[4] = {acc[g][0][2 * h], acc[g][0][2 * h + 1], acc[g][1][2 * h], acc[g][1][2 * h + 1]};  // cc, cc+1, cc+8, cc+9
        if (mode != 1 && bias) {
          o[0] += bias[cc];
          o[1] += bias[cc + 1];
          o[2] += bias[cc + 8];
          o[3] += bias[cc + 9];
        }
        if (mode <= 1) {
          if (mode == 0) {
#pragma unroll
            for (int q = 0; q < 4; q++) o[q] = fmaxf(o[q], 0.f);
          } else if (gate) {
            const __nv_bfloat162 g0 = reinterpret_cast<const __nv_bfloat162 *>(gate + v * NN_CH + cc)[0];
            const __nv_bfloat162 g1 = reinterpret_cast<const __nv_bfloat162 *>(gate + v * NN_CH + cc + 8)[0];
            if (!(__bfloat162float(g0.x) > 0.f)) o[0] = 0.f;
            if (!(__bfloat162float(g0.y) > 0.f)) o[1] = 0.f;
            if (!(__bfloat162float(g1.x) > 0.f)) o[2] = 0.f;
            if (!(__bfloat162float(g1.y) > 0.f)) o[3] = 0.f;
          }
          reinterpret_cast<__nv_bfloat162 *>(Y16 + v * NN_CH + cc)[0] = __floats2bfloat162_rn(o[0], o[1]);
          reinterpret_cast<__nv_bfloat162 *>(Y16 + v * NN_CH + cc + 8)[0] = __floats2bfloat162_rn(o[2], o[3]);
        } else if (cc < 4) {
          if (mode == 2) {
            Y32[v * 4 + cc] = o[0];
            Y32[v * 4 + cc + 1] = o[1];
          } else {
            const int kk = kw + vr + 8 * h;
            const long long gi = ((long long)i * N + j) * P + kk;
            frc[cc * gstride + gi] = o[0];
            if (cc + 1 < 3) frc[(cc + 1) * gstride + gi] = o[1];
          }
        }
      }
    }
  }
}

// Weight and bias gradients, dW[tap][o][c] = sum_v dY[v][o] X[v + d(tap)][c]
// and db[o] = sum_v dY[v][o], over the same tiles as the forward kernel: a
// persistent block stages the 4 x 6 input rows and the 8 dY rows of a tile
// (cp.async, swizzled rows), and warp w owns the three taps dk = 0..2 of
// staged-row offset (di, dj) = (w / 3, w % 3): for each output row it loads
// the dY^T fragments once (ldmatrix.trans) and runs them against the three
// dk-shifted X fragments; warp o < 8 also multiplies output row o's dY^T by a
// ones fragment for the bias.  Sums stay in registers across tiles and are
// written once per block to `partial` [block][NN_WSIZE + 8 x 16]; a second
// kernel adds the blocks in a fixed order (deterministic gradients).
constexpr int kThreadsWg = 32 * 9;
constexpr int kWgPartial = NN_WSIZE + 8 * NN_CH;
constexpr size_t kWgSmem = sizeof(bf16) * ((size_t)CT_ROWS * CT_Q * NN_CH + (size_t)CT_I * CT_J * CT_SEG * NN_CH);

__global__ void __launch_bounds__(kThreadsWg, 3) k_conv_wgrad(const bf16 *__restrict__ X, const bf16 *__restrict__ dY,
                                                              int N, float *__restrict__ partial) {
  extern __shared__ __align__(16) unsigned char wg_smem[];
  bf16(*xs)[CT_Q][NN_CH] = reinterpret_cast<bf16(*)[CT_Q][NN_CH]>(wg_smem);
  bf16(*ys)[CT_SEG][NN_CH] =
      reinterpret_cast<bf16(*)[CT_SEG][NN_CH]>(wg_smem + sizeof(bf16) * (size_t)CT_ROWS * CT_Q * NN_CH);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int rdi = warp / 3, rdj = warp % 3;
  float acc[3][2][4], bacc[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
  for (int t = 0; t < 3; t++)
#pragma unroll
    for (int n = 0; n < 2; n++)
#pragma unroll
      for (int q = 0; q < 4; q++) acc[t][n][q] = 0.f;
  const uint32_t ones = 0x3F803F80u;  // two bf16 1.0
  // ldmatrix.trans lane roles: A = dY^T (16 out x 16 voxels), B = X (16 voxels x 16 in)
  const int a_vox = (lane & 7) + 8 * (lane >> 4), a_half = (lane >> 3) & 1;
  const int b_vox = (lane & 7) + 8 * ((lane >> 3) & 1), b_half = lane >> 4;
  const int nseg = (N + CT_SEG - 1) / CT_SEG, tiles_j = N / CT_J;
  const long long ntiles = (long long)(N / CT_I) * tiles_j * nseg;
  for (long long t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int seg = (int)(t % nseg);
    const long long rest = t / nseg;
    const int i0 = (int)(rest / tiles_j) * CT_I, j0 = (int)(rest % tiles_j) * CT_J, k0 = seg * CT_SEG;
    const int qmax = min(CT_SEG + 1, N - k0 + 1);  // staged voxels past qmax are zero
    __syncthreads();                              // the previous tile's reads are done
    for (int c = tid; c < CT_ROWS * CT_Q * 2; c += kThreadsWg) {
      const int r = c / (CT_Q * 2), rem = c - r * (CT_Q * 2), q = rem >> 1, h = rem & 1;
      bf16 *dst = &xs[r][q][8 * swz_half(q, h)];
      if (q > qmax) {
        *reinterpret_cast<uint4 *>(dst) = make_uint4(0, 0, 0, 0);
        continue;
      }
      int ii = i0 + r / (CT_J + 2) - 1, jj = j0 + r % (CT_J + 2) - 1, kk = k0 - 1 + q;
      ii += ii < 0 ? N : 0;
      ii -= ii >= N ? N : 0;
      jj += jj < 0 ? N : 0;
      jj -= jj >= N ? N : 0;
      kk += kk < 0 ? N : 0;
      kk -= kk >= N ? N : 0;
      cp_async16(dst, X + (((long long)ii * N + jj) * N + kk) * NN_CH + 8 * h);
    }
    for (int c = tid; c < CT_I * CT_J * CT_SEG * 2; c += kThreadsWg) {
      const int o = c / (CT_SEG * 2), rem = c - o * (CT_SEG * 2), q = rem >> 1, h = rem & 1;
      bf16 *dst = &ys[o][q][8 * swz_half(q, h)];
      const int kk = k0 + q;
      if (kk >= N) {
        *reinterpret_cast<uint4 *>(dst) = make_uint4(0, 0, 0, 0);
        continue;
      }
      const int i = i0 + o / CT_J, j = j0 + o % CT_J;
      cp_async16(dst, dY + (((long long)i * N + j) * N + kk) * NN_CH + 8 * h);
    }
    cp_async_wait_all();
    __syncthreads();
    const int ng = min(CT_SEG / 16, (N - k0) / 16);  // 16-voxel steps holding data
    for (int o = 0; o < CT_I * CT_J; o++) {
      const int r = (o / CT_J + rdi) * (CT_J + 2) + (o % CT_J + rdj);
#pragma unroll
      for (int ks = 0; ks < CT_SEG / 16; ks++) {
        if (ks >= ng) break;
        const int qa = 16 * ks + a_vox;
        uint32_t a0, a1, a2, a3;
        ldsm_x4_t(smem_u32(&ys[o][qa][8 * swz_half(qa, a_half)]), a0, a1, a2, a3);
        if (o == warp) mma16816(bacc, a0, a1, a2, a3, ones, ones);
#pragma unroll
        for (int dk = 0; dk < 3; dk++) {
          const int qb = 16 * ks + dk + b_vox;
          uint32_t b0, b1, b2, b3;
          ldsm_x4_t(smem_u32(&xs[r][qb][8 * swz_half(qb, b_half)]), b0, b1, b2, b3);
          mma16816(acc[dk][0], a0, a1, a2, a3, b0, b1);
          mma16816(acc[dk][1], a0, a1, a2, a3, b2, b3);
        }
      }
    }
  }
  // fragment: rows (out) lane/4, lane/4 + 8; columns (in) 2 (lane%4) + {0,1} (+8 for n-tile 1)
  float *pb = partial + (size_t)blockIdx.x * kWgPartial;
  const int o0 = lane >> 2, c0 = 2 * (lane & 3);
#pragma unroll
  for (int dk = 0; dk < 3; dk++) {
    float *w = pb + (3 * warp + dk) * NN_CH * NN_CH;
#pragma unroll
    for (int n = 0; n < 2; n++) {
      w[o0 * NN_CH + c0 + 8 * n] = acc[dk][n][0];
      w[o0 * NN_CH + c0 + 8 * n + 1] = acc[dk][n][1];
      w[(o0 + 8) * NN_CH + c0 + 8 * n] = acc[dk][n][2];
      w[(o0 + 8) * NN_CH + c0 + 8 * n + 1] = acc[dk][n][3];
    }
  }
  if (warp < CT_I * CT_J && (lane & 3) == 0) {  // every column of the ones product holds the row sum
    pb[NN_WSIZE + warp * NN_CH + o0] = bacc[0];
    pb[NN_WSIZE + warp * NN_CH + o0 + 8] = bacc[2];
  }
}

// dW and db from the per-block partial sums in a fixed order: thread row ty
// adds blocks ty, ty + 8, ... in index order, then row 0 adds the 8 row sums
// in order (deterministic gradients).  blockDim (32, 8), 32 outputs a block.
__global__ void k_wgrad_reduce(const float *__restrict__ partial, int nblk, float *__restrict__ dW,
                               float *__restrict__ db) {
  __shared__ float sh[8][32];
  const int tx = threadIdx.x, ty = threadIdx.y, e = blockIdx.x * 32 + tx;
  float s = 0.f;
  if (e < NN_WSIZE) {
    for (int b = ty; b < nblk; b += 8) s += partial[(size_t)b * kWgPartial + e];
  } else if (e < NN_WSIZE + NN_CH) {
    const int c = e - NN_WSIZE;
    for (int b = ty; b < nblk; b += 8)
      for (int w = 0; w < 8; w++) s += partial[(size_t)b * kWgPartial + NN_WSIZE + w * NN_CH + c];
  }
  sh[ty][tx] = s;
  __syncthreads();
  if (ty == 0) {
    float t = 0.f;
    for (int r = 0; r < 8; r++) t += sh[r][tx];
    if (e < NN_WSIZE) dW[e] = t;
    else if (e < NN_WSIZE + NN_CH) db[e - NN_WSIZE] = t;
  }
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
    rowv[1] = __float2bfloat16_rn(ph * 1e5f);
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

// Training-set compaction: 3 feature channels (bf16) and, for grid targets,
// 3 target components (f32) per voxel (dt / t NULL: features only).
__global__ void k_pack_sample(const bf16 *__restrict__ X, const float *__restrict__ t, long long V,
                              bf16 *__restrict__ dx, float *__restrict__ dt) {
  long long stride = (long long)gridDim.x * blockDim.x;
  for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < V; v += stride)
#pragma unroll
    for (int c = 0; c < 3; c++) {
      dx[v * 3 + c] = X[v * NN_CH + c];
      if (dt) dt[v * 3 + c] = t[v * 4 + c];
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
    for (int c = 0; c < 3; c++) rowv[c] = dx[v * 3 + c];
    if (dt) {
#pragma unroll
      for (int c = 0; c < 3; c++) t[v * 4 + c] = dt[v * 3 + c];
      t[v * 4 + 3] = 0.f;
    }
    reinterpret_cast<uint4 *>(X + v * NN_CH)[0] = reinterpret_cast<uint4 *>(rowv)[0];
    reinterpret_cast<uint4 *>(X + v * NN_CH)[1] = reinterpret_cast<uint4 *>(rowv)[1];
  }
}

// Trilinear (CIC) interpolation of three force grids at a cell position, the
// gather of the kick (MtoParticles, src/auxPM.c:560-644).
__device__ __forceinline__ void cic_gather3(const float *__restrict__ F, long long gf, int N, long long P, int ix,
                                            int iy, int iz, float dx, float dy, float dz, float out[3]) {
  const long long NP = (long long)N * P;
  const long long x0 = (long long)ix * NP, x1 = (ix + 1 == N ? 0 : (long long)(ix + 1) * NP);
  const long long y0 = (long long)iy * P, y1 = (iy + 1 == N ? 0 : (long long)(iy + 1) * P);
  const long long z0 = iz, z1 = (iz + 1 == N ? 0 : iz + 1);
  const float tx = 1.f - dx, ty = 1.f - dy, tz = 1.f - dz;
#pragma unroll
  for (int q = 0; q < 3; q++) {
    const float *G = F + q * gf;
    out[q] = G[x0 + y0 + z0] * (tx * ty * tz) + G[x0 + y0 + z1] * (tx * ty * dz) + G[x0 + y1 + z0] * (tx * dy * tz) +
             G[x0 + y1 + z1] * (tx * dy * dz) + G[x1 + y0 + z0] * (dx * ty * tz) + G[x1 + y0 + z1] * (dx * ty * dz) +
             G[x1 + y1 + z0] * (dx * dy * tz) + G[x1 + y1 + z1] * (dx * dy * dz);
  }
}

// Particle-level target: per particle, the fine context's interpolated force
// minus the coarse context's (each at its own copy of the particle), and the
// particle's coarse-mesh cell coordinates (cell + CIC fraction), SoA [3][np].
__global__ void k_particle_target(const float *__restrict__ ff, long long fg, int Nf, long long Pf,
                                  const float *__restrict__ sf, const mgp_dstate *__restrict__ stf,
                                  const float *__restrict__ fc, long long cg, int N, long long P,
                                  const float *__restrict__ sc, const mgp_dstate *__restrict__ stc, long long np,
                                  int Ns, float scale_f, float scale_c, float *__restrict__ pc,
                                  float *__restrict__ pt) {
  const float oxf = (float)(stf->cx[0] * scale_f), oyf = (float)(stf->cx[1] * scale_f),
              ozf = (float)(stf->cx[2] * scale_f);
  const float oxc = (float)(stc->cx[0] * scale_c), oyc = (float)(stc->cx[1] * scale_c),
              ozc = (float)(stc->cx[2] * scale_c);
  long long stride = (long long)gridDim.x * blockDim.x;
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < np; p += stride) {
    int i, j, k, ix, iy, iz;
    float dx, dy, dz, Ff[3], Fc[3];
    lattice_ijk(p, Ns, i, j, k);
    cell_frac(i, sf[p], oxf, Nf, Ns, scale_f, ix, dx);
    cell_frac(j, sf[np + p], oyf, Nf, Ns, scale_f, iy, dy);
    cell_frac(k, sf[2 * np + p], ozf, Nf, Ns, scale_f, iz, dz);
    cic_gather3(ff, fg, Nf, Pf, ix, iy, iz, dx, dy, dz, Ff);
    cell_frac(i, sc[p], oxc, N, Ns, scale_c, ix, dx);
    cell_frac(j, sc[np + p], oyc, N, Ns, scale_c, iy, dy);
    cell_frac(k, sc[2 * np + p], ozc, N, Ns, scale_c, iz, dz);
    cic_gather3(fc, cg, N, P, ix, iy, iz, dx, dy, dz, Fc);
    pc[p] = (float)ix + dx;
    pc[np + p] = (float)iy + dy;
    pc[2 * np + p] = (float)iz + dz;
#pragma unroll
    for (int q = 0; q < 3; q++) pt[q * np + p] = Ff[q] - Fc[q];
  }
}

// Particle loss = sum over particles and components of (s u_p - r_p)^2 / (3 np),
// u_p the CIC interpolation at the particle of the (high-passed) network
// output, held as three padded real grids (grid c at u + c gstride, rows of
// P floats); its gradient d loss / d u is the CIC deposit of
// 2 s (s u_p - r_p) / (3 np), accumulated per voxel into dacc [V][4] with one
// float4 atomic per corner.
constexpr int kThreadsPl = 256;
__global__ void __launch_bounds__(kThreadsPl) k_particle_loss(const float *__restrict__ u, long long gstride, long long P,
                                                              int N, long long np, const float *__restrict__ pc,
                                                              const float *__restrict__ pt, float s, float inv,
                                                              float *__restrict__ dacc, double *__restrict__ loss) {
  __shared__ double sh[kThreadsPl / 32];
  double acc = 0.0;
  long long stride = (long long)gridDim.x * blockDim.x;
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < np; p += stride) {
    int i0[3], i1[3];
    float d[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
      const float w = pc[a * np + p], fl = floorf(w);
      d[a] = w - fl;
      int ic = (int)fl % N;
      if (ic < 0) ic += N;
      i0[a] = ic;
      i1[a] = ic + 1 == N ? 0 : ic + 1;
    }
    long long g[8], vx[8];
    float wt[8];
#pragma unroll
    for (int c = 0; c < 8; c++) {
      const int bx = c >> 2, by = (c >> 1) & 1, bz = c & 1;
      const long long row = (long long)(bx ? i1[0] : i0[0]) * N + (by ? i1[1] : i0[1]);
      g[c] = row * P + (bz ? i1[2] : i0[2]);
      vx[c] = row * N + (bz ? i1[2] : i0[2]);
      wt[c] = (bx ? d[0] : 1.f - d[0]) * (by ? d[1] : 1.f - d[1]) * (bz ? d[2] : 1.f - d[2]);
    }
    float e[3];
#pragma unroll
    for (int q = 0; q < 3; q++) {
      float uq = 0.f;
#pragma unroll
      for (int c = 0; c < 8; c++) uq = fmaf(wt[c], __ldg(u + q * gstride + g[c]), uq);
      e[q] = s * uq - pt[q * np + p];
      acc += (double)e[q] * e[q];
    }
    const float gs = 2.f * s * inv;
#pragma unroll
    for (int c = 0; c < 8; c++) {
      const float gw = gs * wt[c];
      atomicAdd(reinterpret_cast<float4 *>(dacc) + vx[c], make_float4(gw * e[0], gw * e[1], gw * e[2], 0.f));
    }
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < kThreadsPl / 32; w++) t += sh[w];
    atomicAdd(loss, t * (double)inv);
  }
}

// dacc [V][4] (channels 0-2) -> three padded real grids.
__global__ void k_acc4_to_grids(const float *__restrict__ dacc, int N, long long P, long long gstride,
                                float *__restrict__ du) {
  const long long V = (long long)N * N * N;
  long long stride = (long long)gridDim.x * blockDim.x;
  for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < V; v += stride) {
    const long long row = v / N;
    const long long gi = row * P + (v - row * N);
    const float4 a = reinterpret_cast<const float4 *>(dacc)[v];
    du[gi] = a.x;
    du[gstride + gi] = a.y;
    du[2 * gstride + gi] = a.z;
  }
}

// Three padded real grids (channels 0-2) -> the BF16 gradient [V][16] of the
// last layer.
__global__ void k_grids_to_bf16(const float *__restrict__ du, long long gstride, long long P, int N,
                                bf16 *__restrict__ g) {
  const long long V = (long long)N * N * N;
  long long stride = (long long)gridDim.x * blockDim.x;
  for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < V; v += stride) {
    const long long row = v / N;
    const long long gi = row * P + (v - row * N);
    __align__(16) bf16 r[NN_CH];
#pragma unroll
    for (int c = 0; c < NN_CH; c++) r[c] = __float2bfloat16_rn(0.f);
    r[0] = __float2bfloat16_rn(du[gi]);
    r[1] = __float2bfloat16_rn(du[gstride + gi]);
    r[2] = __float2bfloat16_rn(du[2 * gstride + gi]);
    reinterpret_cast<uint4 *>(g + v * NN_CH)[0] = reinterpret_cast<uint4 *>(r)[0];
    reinterpret_cast<uint4 *>(g + v * NN_CH)[1] = reinterpret_cast<uint4 *>(r)[1];
  }
}

// Sharp high-pass of three transformed grids (complex [N][N][N/2+1] each,
// grid c at src + c cstride): modes with wavelength N / |n| >= lambda cells
// (n the integer wave vector) are zeroed, the others scaled by `factor`;
// added to dst (the force transforms) when dst is given, else in place.
__global__ void k_highpass(float2 *__restrict__ src, long long cstride, int N, float lambda, float factor,
                           float2 *__restrict__ dst) {
  const int NH = N / 2 + 1;
  const long long n = (long long)N * N * NH;
  const float kc2 = lambda > 0.f ? ((float)N / lambda) * ((float)N / lambda) : 0.f;  // |n|^2 kept from here
  long long stride = (long long)gridDim.x * blockDim.x;
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += stride) {
    const int kz = (int)(q % NH);
    const long long r = q / NH;
    const int j = (int)(r % N), i = (int)(r / N);
    const int ki = i <= N / 2 ? i : i - N, kj = j <= N / 2 ? j : j - N;
    const float k2 = (float)(ki * ki + kj * kj + kz * kz);
    const float h = (k2 > 0.f && k2 > kc2) ? factor : 0.f;
#pragma unroll
    for (int c = 0; c < 3; c++) {
      const float2 v = src[c * cstride + q];
      if (dst) {
        float2 o = dst[c * cstride + q];
        o.x += h * v.x;
        o.y += h * v.y;
        dst[c * cstride + q] = o;
      } else {
        src[c * cstride + q] = make_float2(h * v.x, h * v.y);
      }
    }
  }
}

// Keep the modes of a fine-mesh transform [Nf][Nf][Nf/2+1] that the coarse
// mesh represents (|k_x|, |k_y|, k_z < kc in fine integer units), scaled by
// norm (the 1/Nf^3 of the round trip); zero the rest.
__global__ void k_band_limit(float2 *__restrict__ c, int Nf, int kc, float norm) {
  const int NH = Nf / 2 + 1;
  const long long n = (long long)Nf * Nf * NH;
  long long stride = (long long)gridDim.x * blockDim.x;
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += stride) {
    const int kz = (int)(q % NH);
    const long long r = q / NH;
    const int j = (int)(r % Nf), i = (int)(r / Nf);
    const int ki = i < Nf / 2 ? i : Nf - i, kj = j < Nf / 2 ? j : Nf - j;
    const float f = (ki < kc && kj < kc && kz < kc) ? norm : 0.f;
    float2 v = c[q];
    v.x *= f;
    v.y *= f;
    c[q] = v;
  }
}

// sum of squares of n floats into *out (FP64)
__global__ void k_sumsq_flat(const float *__restrict__ a, long long n, double *__restrict__ out) {
  __shared__ double sh[8];
  double acc = 0.0;
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x)
    acc += (double)a[q] * a[q];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += sh[w];
    atomicAdd(out, t);
  }
}

}  // namespace

// --------------------------------------------------------------- host side
#define NN_RET(x)                  \
  do {                             \
    int rc_ = (x);                 \
    if (rc_ != MGP_OK) return rc_; \
  } while (0)

// Output / gradient grids and the closure's own transforms (lazy).
static int ensure_hp(mgp_closure *cl) {
  const long long gf = (long long)cl->N * cl->N * cl->P;
  if (!cl->ugrid) MGP_CUDA(cudaMalloc(&cl->ugrid, sizeof(float) * 3 * gf));
  if (!cl->dgrid) MGP_CUDA(cudaMalloc(&cl->dgrid, sizeof(float) * 3 * gf));
  if (!cl->have_plans) {
    long long n[3] = {cl->N, cl->N, cl->N};
    long long rembed[3] = {cl->N, cl->N, cl->P}, cembed[3] = {cl->N, cl->N, cl->P / 2};
    const long long rdist = gf, cdist = gf / 2;
    size_t ws = 0;
    MGP_CUFFT(cufftCreate(&cl->plan_r2c));
    MGP_CUFFT(cufftCreate(&cl->plan_c2r));
    cl->have_plans = 1;
    MGP_CUFFT(cufftMakePlanMany64(cl->plan_r2c, 3, n, rembed, 1, rdist, cembed, 1, cdist, CUFFT_R2C, 1, &ws));
    MGP_CUFFT(cufftMakePlanMany64(cl->plan_c2r, 3, n, cembed, 1, cdist, rembed, 1, rdist, CUFFT_C2R, 1, &ws));
  }
  return MGP_OK;
}

// In place: the three grids at g become their high-pass (R2C, filter with
// the 1/N^3 of the round trip, C2R) on stream st.
static int highpass_grids(mgp_closure *cl, float *g, cudaStream_t st) {
  const long long gf = (long long)cl->N * cl->N * cl->P;
  MGP_CUFFT(cufftSetStream(cl->plan_r2c, st));
  MGP_CUFFT(cufftSetStream(cl->plan_c2r, st));
  for (int c = 0; c < 3; c++)
    MGP_CUFFT(cufftExecR2C(cl->plan_r2c, (cufftReal *)(g + c * gf), (cufftComplex *)(g + c * gf)));
  k_highpass<<<mgp_blocks_for(gf / 2, 4), 256, 0, st>>>((float2 *)g, gf / 2, cl->N, cl->hp_lambda,
                                                      (float)(1.0 / ((double)cl->V)), NULL);
  MGP_CHECK_LAUNCH();
  g_kernel_launches++;
  for (int c = 0; c < 3; c++)
    MGP_CUFFT(cufftExecC2R(cl->plan_c2r, (cufftComplex *)(g + c * gf), (cufftReal *)(g + c * gf)));
  return MGP_OK;
}

static int conv_fwd(mgp_closure *cl, const bf16 *X, const bf16 *W, const float *bias, const bf16 *gate, int mode,
                    bf16 *Y16, float *Y32,
                    float *frc, long long gstride, long long P, float scale) {
  static int grid = 0;  // resident CTAs of the persistent kernel (one device per process)
  if (!grid) {
    MGP_CUDA(cudaFuncSetAttribute(k_conv_fwd, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kConvSmem));
    int per_sm = 0, sms = 0;
    MGP_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_conv_fwd, kThreadsConv, kConvSmem));
    MGP_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, cl->device));
    grid = sms * (per_sm > 0 ? per_sm : 1);
  }
  const int N = cl->N;
  const long long tiles = (long long)(N / CT_I) * (N / CT_J) * ((N + CT_SEG - 1) / CT_SEG);
  const unsigned blocks = (unsigned)(tiles < grid ? tiles : grid);
  k_conv_fwd<<<blocks, kThreadsConv, kConvSmem, cl->stream>>>(X, W, bias, gate, N, mode, Y16, Y32, frc, gstride, P,
                                                              scale);
  MGP_CHECK_LAUNCH();
  g_kernel_launches++;
  return MGP_OK;
}

static int conv_wgrad(mgp_closure *cl, const bf16 *X, const bf16 *dY, float *dW, float *db) {
  static int grid = 0;  // resident blocks of the persistent kernel (one device per process)
  if (!grid) {
    MGP_CUDA(cudaFuncSetAttribute(k_conv_wgrad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kWgSmem));
    MGP_CUDA(cudaFuncSetAttribute(k_conv_wgrad, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
    int per_sm = 0, sms = 0;
    MGP_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_conv_wgrad, kThreadsWg, kWgSmem));
    MGP_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, cl->device));
    grid = sms * (per_sm > 0 ? per_sm : 1);
  }
  const int N = cl->N;
  const long long tiles = (long long)(N / CT_I) * (N / CT_J) * ((N + CT_SEG - 1) / CT_SEG);
  const int blocks = (int)(tiles < grid ? tiles : grid);
  if (cl->wg_blocks < blocks) {
    if (cl->wg_partial) cudaFree(cl->wg_partial);
    cl->wg_partial = NULL;
    cl->wg_blocks = 0;
    MGP_CUDA(cudaMalloc(&cl->wg_partial, sizeof(float) * (size_t)kWgPartial * blocks));
    cl->wg_blocks = blocks;
  }
  k_conv_wgrad<<<blocks, kThreadsWg, kWgSmem, cl->stream>>>(X, dY, N, cl->wg_partial);
  MGP_CHECK_LAUNCH();
  k_wgrad_reduce<<<(NN_WSIZE + NN_CH + 31) / 32, dim3(32, 8), 0, cl->stream>>>(cl->wg_partial, blocks, dW, db);
  MGP_CHECK_LAUNCH();
  g_kernel_launches += 2;
  return MGP_OK;
}

// Forward pass; grid = 0: raw output into out [V][4]; grid = 1: the
// high-passed output into ugrid (the particle loss and the in-step path).
static int closure_forward(mgp_closure *cl, int grid) {
  for (int l = 0; l < NN_LAYERS - 1; l++)
    NN_RET(conv_fwd(cl, cl->act[l], cl->w16[l], cl->b32[l], NULL, 0, cl->act[l + 1], NULL, NULL, 0, 0, 0.f));
  if (grid) {
    NN_RET(ensure_hp(cl));
    NN_RET(conv_fwd(cl, cl->act[NN_LAYERS - 1], cl->w16[NN_LAYERS - 1], cl->b32[NN_LAYERS - 1], NULL, 3, NULL, NULL,
                    cl->ugrid, (long long)cl->N * cl->N * cl->P, cl->P, 0.f));
    return highpass_grids(cl, cl->ugrid, cl->stream);
  }
  return conv_fwd(cl, cl->act[NN_LAYERS - 1], cl->w16[NN_LAYERS - 1], cl->b32[NN_LAYERS - 1], NULL, 2, NULL, cl->out,
                  NULL,
                  0, 0, 0.f);
}

// Loss and all gradients for the current features/target.
static int closure_backward(mgp_closure *cl) {
  const long long V = cl->V;
  MGP_CUDA(cudaMemsetAsync(cl->loss, 0, sizeof(double), cl->stream));
  if (cl->pmode) {
    const long long gf = (long long)cl->N * cl->N * cl->P;
    MGP_CUDA(cudaMemsetAsync(cl->out, 0, sizeof(float) * 4 * V, cl->stream));  // the deposit's accumulator
    k_particle_loss<<<mgp_blocks_for(cl->np, 8), kThreadsPl, 0, cl->stream>>>(
        cl->ugrid, gf, cl->P, cl->N, cl->np, cl->cur_pc, cl->cur_pt, cl->pnorm ? cl->pscale : cl->out_scale,
        (float)(1.0 / (3.0 * (double)cl->np * (cl->pnorm ? (double)cl->pscale * cl->pscale : 1.0))), cl->out,
        cl->loss);
    MGP_CHECK_LAUNCH();
    k_acc4_to_grids<<<mgp_blocks_for(V, 4), 256, 0, cl->stream>>>(cl->out, cl->N, cl->P, gf, cl->dgrid);
    MGP_CHECK_LAUNCH();
    g_kernel_launches += 2;
    NN_RET(highpass_grids(cl, cl->dgrid, cl->stream));  // the filter is symmetric: its adjoint is itself
    k_grids_to_bf16<<<mgp_blocks_for(V, 4), 256, 0, cl->stream>>>(cl->dgrid, gf, cl->P, cl->N, cl->g0);
    MGP_CHECK_LAUNCH();
    g_kernel_launches++;
  } else {
    k_loss_grad<<<mgp_blocks_for(V, 4), 256, 0, cl->stream>>>(cl->out, cl->target, V, cl->out_scale, cl->g0, cl->loss);
    MGP_CHECK_LAUNCH();
    g_kernel_launches++;
  }
  bf16 *g = cl->g0, *gn = cl->g1;
  for (int l = NN_LAYERS - 1; l >= 0; l--) {
    NN_RET(conv_wgrad(cl, cl->act[l], g, cl->gw[l], cl->gb[l]));
    if (l == 0) break;
    k_mirror_transpose<<<(NN_WSIZE + 255) / 256, 256, 0, cl->stream>>>(cl->w16[l], cl->wt16);
    MGP_CHECK_LAUNCH();
    g_kernel_launches++;
    NN_RET(conv_fwd(cl, g, cl->wt16, NULL, cl->act[l], 1, gn, NULL, NULL, 0, 0, 0.f));
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
  void *b[] = {cl->wt16, cl->out,  cl->target, cl->g0,   cl->g1,   cl->loss,  cl->grid_a, cl->grid_b,
               cl->ds_x, cl->ds_t, cl->ds_pc,  cl->ds_pt, cl->pc,   cl->pt,    cl->ugrid, cl->dgrid, cl->fscr,
               cl->wg_partial};
  for (size_t q = 0; q < sizeof(b) / sizeof(b[0]); q++)
    if (b[q]) cudaFree(b[q]);
  if (cl->have_plans) {
    cufftDestroy(cl->plan_r2c);
    cufftDestroy(cl->plan_c2r);
  }
  if (cl->own_stream && cl->stream) cudaStreamDestroy(cl->stream);
  free(cl->ds_s);
  free(cl->scale_a);
  free(cl->scale_s);
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
  cl->hp_lambda = 0.0f;
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
      for (auto &x : w) x = 0.f;  // start at the plain PM force (zero residual)
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
    cl->pmode = 0;
  }
  return MGP_OK;
}

// Forward pass on the working features; out [V][3] host (may be NULL).
extern "C" int mgp_closure_forward(mgp_closure *cl, float *out) {
  if (!cl) return mgp_set_error(MGP_EINVAL, "null closure");
  MGP_CUDA(cudaSetDevice(cl->device));
  NN_RET(closure_forward(cl, 0));
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
  NN_RET(closure_forward(cl, cl->pmode));
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
  NN_RET(closure_forward(cl, cl->pmode));
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
  cl->pmode = 0;
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

// Particle buffers (SoA [3][np]) and the f32 gradient grid for np particles.
static int ensure_particles(mgp_closure *cl, long long np) {
  if (np <= 0) return mgp_set_error(MGP_EINVAL, "particle sample needs np > 0");
  if (cl->own_np != np) {
    if (cl->pc) cudaFree(cl->pc);
    if (cl->pt) cudaFree(cl->pt);
    cl->pc = cl->pt = NULL;
    cl->own_np = 0;
    MGP_CUDA(cudaMalloc(&cl->pc, sizeof(float) * 3 * np));
    MGP_CUDA(cudaMalloc(&cl->pt, sizeof(float) * 3 * np));
    cl->own_np = np;
  }
  cl->np = np;
  return ensure_hp(cl);
}

// Particle-level training target from a fine and a coarse context holding the
// same particles, both after mgp_get_displacements at the same scale factor.
// band != 0: the fine force is first restricted to the modes the coarse mesh
// represents (three R2C / C2R pairs on the fine mesh), which drops the
// sub-grid force that no coarse-mesh input can predict.
extern "C" int mgp_closure_target_particles(mgp_closure *cl, mgp_ctx *fine, mgp_ctx *coarse, int band,
                                            double *rms) {
  NN_RET(check_ctx(cl, coarse));
  if (!fine || fine->nbox != 1 || !fine->have_forces) return mgp_set_error(MGP_ESTATE, "fine context has no forces");
  if (fine->np != coarse->np || fine->Ns != coarse->Ns || fine->p.Box != coarse->p.Box)
    return mgp_set_error(MGP_EINVAL, "fine and coarse contexts hold different particle sets");
  MGP_CUDA(cudaSetDevice(cl->device));
  // both particle sets in lattice order (the sample pairs them by index)
  NN_RET(mgp_particles_canonical(fine));
  NN_RET(mgp_particles_canonical(coarse));
  MGP_CUDA(cudaStreamSynchronize(fine->stream));
  MGP_CUDA(cudaStreamSynchronize(coarse->stream));
  NN_RET(ensure_particles(cl, coarse->np));
  const float *ff = fine->frc;
  if (band) {
    const long long gf = fine->g.nreal;
    if (cl->fscr_floats != 3 * gf) {
      if (cl->fscr) cudaFree(cl->fscr);
      cl->fscr = NULL;
      cl->fscr_floats = 0;
      MGP_CUDA(cudaMalloc(&cl->fscr, sizeof(float) * 3 * gf));
      cl->fscr_floats = 3 * gf;
    }
    MGP_CUDA(cudaMemcpyAsync(cl->fscr, fine->frc, sizeof(float) * 3 * gf, cudaMemcpyDeviceToDevice, cl->stream));
    MGP_CUFFT(cufftSetStream(fine->plan_r2c_ip, cl->stream));
    MGP_CUFFT(cufftSetStream(fine->plan_c2r_1, cl->stream));
    const int Nf = fine->g.N;
    cufftResult r = CUFFT_SUCCESS;
    for (int q = 0; q < 3 && r == CUFFT_SUCCESS; q++) {
      float *g = cl->fscr + q * gf;
      r = cufftExecR2C(fine->plan_r2c_ip, (cufftReal *)g, (cufftComplex *)g);
      if (r != CUFFT_SUCCESS) break;
      k_band_limit<<<mgp_blocks_for(fine->g.ncomplex, 4), 256, 0, cl->stream>>>(
          (float2 *)g, Nf, coarse->g.N / 2, (float)(1.0 / ((double)Nf * Nf * Nf)));
      g_kernel_launches++;
      r = cufftExecC2R(fine->plan_c2r_1, (cufftComplex *)g, (cufftReal *)g);
    }
    cufftSetStream(fine->plan_r2c_ip, fine->stream);
    cufftSetStream(fine->plan_c2r_1, fine->stream);
    if (r != CUFFT_SUCCESS) return mgp_set_error(MGP_ECUFFT, "closure band-limited target transforms");
    MGP_CHECK_LAUNCH();
    ff = cl->fscr;
  }
  const double box = coarse->p.Box;
  k_particle_target<<<mgp_blocks_for(cl->np, 8), 256, 0, cl->stream>>>(
      ff, fine->g.nreal, fine->g.N, fine->g.P, fine->s, fine->dstate, coarse->frc, coarse->g.nreal,
      coarse->g.N, coarse->g.P, coarse->s, coarse->dstate, cl->np, coarse->Ns, (float)(fine->g.N / box),
      (float)(coarse->g.N / box), cl->pc, cl->pt);
  MGP_CHECK_LAUNCH();
  g_kernel_launches++;
  cl->cur_pc = cl->pc;
  cl->cur_pt = cl->pt;
  cl->pmode = 1;
  // The sample trains the network to predict its residual in units of its
  // own rms (the residual grows ~200x over a run, and an unnormalised loss
  // leaves the early steps, whose errors grow the most, unconstrained).
  MGP_CUDA(cudaMemsetAsync(cl->loss, 0, sizeof(double), cl->stream));
  k_sumsq_flat<<<mgp_blocks_for(3 * cl->np, 4), 256, 0, cl->stream>>>(cl->pt, 3 * cl->np, cl->loss);
  MGP_CHECK_LAUNCH();
  double ss = 0.0;
  MGP_CUDA(cudaMemcpyAsync(&ss, cl->loss, sizeof(double), cudaMemcpyDeviceToHost, cl->stream));
  MGP_CUDA(cudaStreamSynchronize(cl->stream));
  const double r = sqrt(ss / (3.0 * (double)cl->np));
  cl->pscale = r > 0.0 ? (float)r : 1.0f;
  cl->pnorm = 1;
  if (rms) *rms = r;
  MGP_CUDA(cudaStreamSynchronize(cl->stream));
  return MGP_OK;
}

// Host particle sample: cells [np][3] (mesh units, [0, Nmesh)), t [np][3].
extern "C" int mgp_closure_set_particle_sample(mgp_closure *cl, long long np, const float *cells, const float *t) {
  if (!cl || !cells || !t) return mgp_set_error(MGP_EINVAL, "null argument");
  for (long long q = 0; q < 3 * np; q++)
    if (!(cells[q] >= 0.f && cells[q] < (float)cl->N))
      return mgp_set_error(MGP_EINVAL, "particle cell coordinate %g outside [0, %d)", cells[q], cl->N);
  MGP_CUDA(cudaSetDevice(cl->device));
  MGP_CUDA(cudaStreamSynchronize(cl->stream));
  NN_RET(ensure_particles(cl, np));
  std::vector<float> hc((size_t)3 * np), ht((size_t)3 * np);
  for (long long p = 0; p < np; p++)
    for (int a = 0; a < 3; a++) {
      hc[a * np + p] = cells[p * 3 + a];
      ht[a * np + p] = t[p * 3 + a];
    }
  MGP_CUDA(cudaMemcpy(cl->pc, hc.data(), sizeof(float) * hc.size(), cudaMemcpyHostToDevice));
  MGP_CUDA(cudaMemcpy(cl->pt, ht.data(), sizeof(float) * ht.size(), cudaMemcpyHostToDevice));
  cl->cur_pc = cl->pc;
  cl->cur_pt = cl->pt;
  cl->pmode = 1;
  cl->pnorm = 0;  // a host sample uses out_scale and an unnormalised loss
  return MGP_OK;
}

extern "C" int mgp_closure_get_particle_sample(mgp_closure *cl, long long *np, float *cells, float *t) {
  if (!cl) return mgp_set_error(MGP_EINVAL, "null closure");
  if (np) *np = cl->pmode ? cl->np : 0;
  if (!cl->pmode) return MGP_OK;
  MGP_CUDA(cudaStreamSynchronize(cl->stream));
  const long long n = cl->np;
  std::vector<float> hc((size_t)3 * n), ht((size_t)3 * n);
  MGP_CUDA(cudaMemcpy(hc.data(), cl->cur_pc, sizeof(float) * hc.size(), cudaMemcpyDeviceToHost));
  MGP_CUDA(cudaMemcpy(ht.data(), cl->cur_pt, sizeof(float) * ht.size(), cudaMemcpyDeviceToHost));
  for (long long p = 0; p < n; p++)
    for (int a = 0; a < 3; a++) {
      if (cells) cells[p * 3 + a] = hc[a * n + p];
      if (t) t[p * 3 + a] = ht[a * n + p];
    }
  return MGP_OK;
}

// Training set on the device: `n` slots of 3 feature channels per voxel and
// either grid targets (np = 0) or particle samples of np particles.
extern "C" int mgp_closure_reserve(mgp_closure *cl, int n, long long np) {
  if (!cl || n < 0 || np < 0) return mgp_set_error(MGP_EINVAL, "bad closure reserve");
  MGP_CUDA(cudaSetDevice(cl->device));
  MGP_CUDA(cudaStreamSynchronize(cl->stream));
  void *b[] = {cl->ds_x, cl->ds_t, cl->ds_pc, cl->ds_pt};
  for (size_t q = 0; q < sizeof(b) / sizeof(b[0]); q++)
    if (b[q]) cudaFree(b[q]);
  cl->ds_x = NULL;
  cl->ds_t = cl->ds_pc = cl->ds_pt = NULL;
  cl->cap_samples = cl->nsamples = 0;
  cl->ds_np = 0;
  free(cl->ds_s);
  cl->ds_s = NULL;
  if (cl->pmode && cl->cur_pc != cl->pc) cl->pmode = 0;  // the working sample pointed into the old set
  if (n == 0) return MGP_OK;
  MGP_CUDA(cudaMalloc(&cl->ds_x, sizeof(bf16) * 3 * cl->V * n));
  if (np > 0) {
    MGP_CUDA(cudaMalloc(&cl->ds_pc, sizeof(float) * 3 * np * n));
    MGP_CUDA(cudaMalloc(&cl->ds_pt, sizeof(float) * 3 * np * n));
  } else {
    MGP_CUDA(cudaMalloc(&cl->ds_t, sizeof(float) * 3 * cl->V * n));
  }
  cl->ds_s = (float *)calloc(2 * (size_t)n, sizeof(float));  // scale, normalisation flag
  if (!cl->ds_s) return mgp_set_error(MGP_ENOMEM, "closure sample scales");
  cl->ds_np = np;
  cl->cap_samples = n;
  return MGP_OK;
}

extern "C" int mgp_closure_store(mgp_closure *cl, int slot) {
  if (!cl || slot < 0 || slot >= cl->cap_samples) return mgp_set_error(MGP_EINVAL, "bad closure slot %d", slot);
  if (cl->ds_np ? !(cl->pmode && cl->np == cl->ds_np) : cl->pmode)
    return mgp_set_error(MGP_ESTATE, "working sample does not match the reserved set (particles %lld vs %lld)",
                         cl->pmode ? cl->np : 0LL, cl->ds_np);
  k_pack_sample<<<mgp_blocks_for(cl->V, 4), 256, 0, cl->stream>>>(
      cl->act[0], cl->target, cl->V, cl->ds_x + (size_t)slot * 3 * cl->V,
      cl->ds_np ? NULL : cl->ds_t + (size_t)slot * 3 * cl->V);
  MGP_CHECK_LAUNCH();
  if (cl->ds_np) {
    const size_t n3 = (size_t)3 * cl->ds_np;
    MGP_CUDA(cudaMemcpyAsync(cl->ds_pc + slot * n3, cl->cur_pc, sizeof(float) * n3, cudaMemcpyDeviceToDevice,
                             cl->stream));
    MGP_CUDA(cudaMemcpyAsync(cl->ds_pt + slot * n3, cl->cur_pt, sizeof(float) * n3, cudaMemcpyDeviceToDevice,
                             cl->stream));
  }
  cl->ds_s[2 * slot] = cl->pmode && cl->pnorm ? cl->pscale : 0.f;
  cl->ds_s[2 * slot + 1] = cl->pmode ? (float)cl->pnorm : 0.f;
  if (slot >= cl->nsamples) cl->nsamples = slot + 1;
  MGP_CUDA(cudaStreamSynchronize(cl->stream));
  return MGP_OK;
}

// Make a stored slot the working sample (particle samples are used in place).
extern "C" int mgp_closure_load(mgp_closure *cl, int slot) {
  if (!cl || slot < 0 || slot >= cl->nsamples) return mgp_set_error(MGP_EINVAL, "bad closure slot %d", slot);
  k_unpack_sample<<<mgp_blocks_for(cl->V, 4), 256, 0, cl->stream>>>(
      cl->ds_x + (size_t)slot * 3 * cl->V, cl->ds_np ? NULL : cl->ds_t + (size_t)slot * 3 * cl->V, cl->V,
      cl->act[0], cl->target);
  MGP_CHECK_LAUNCH();
  if (cl->ds_np) {
    NN_RET(ensure_hp(cl));
    const size_t n3 = (size_t)3 * cl->ds_np;
    cl->np = cl->ds_np;
    cl->cur_pc = cl->ds_pc + slot * n3;
    cl->cur_pt = cl->ds_pt + slot * n3;
    cl->pmode = 1;
    cl->pscale = cl->ds_s[2 * slot];
    cl->pnorm = cl->ds_s[2 * slot + 1] != 0.f;
  } else {
    cl->pmode = 0;
  }
  return MGP_OK;
}

// Output scale at scale factor A: log-log interpolation of the residual-scale
// table (held at its end values outside it), or out_scale without a table.
static double closure_scale(const mgp_closure *cl, double A) {
  const int n = cl->scale_n;
  if (n <= 0) return cl->out_scale;
  if (n == 1 || A <= cl->scale_a[0]) return cl->scale_s[0];
  if (A >= cl->scale_a[n - 1]) return cl->scale_s[n - 1];
  int q = 0;
  while (q < n - 2 && A > cl->scale_a[q + 1]) q++;
  const double t = log(A / cl->scale_a[q]) / log(cl->scale_a[q + 1] / cl->scale_a[q]);
  return exp((1.0 - t) * log(cl->scale_s[q]) + t * log(cl->scale_s[q + 1]));
}

// Inference inside a PM step, called by mgp_get_displacements between the
// force pass and the force C2R: features, four layers (the last into the
// three output grids), their R2C, and out_scale * H(k) / N^3 times them
// added to the three force transforms, so the context's C2R yields the PM
// force plus the high-passed closure force; all on the context's stream.
int mgp_closure_apply(mgp_closure *cl, mgp_ctx *c, double A) {
  cudaStream_t keep = cl->stream;
  cl->stream = c->stream;
  int rc = ensure_hp(cl);
  if (rc == MGP_OK) rc = closure_features(cl, c, A);
  mgp_tstart(c, T_NNCONV);  // the four convolutions
  for (int l = 0; l < NN_LAYERS - 1 && rc == MGP_OK; l++)
    rc = conv_fwd(cl, cl->act[l], cl->w16[l], cl->b32[l], NULL, 0, cl->act[l + 1], NULL, NULL, 0, 0, 0.f);
  const long long gf = (long long)cl->N * cl->N * cl->P;
  if (rc == MGP_OK)
    rc = conv_fwd(cl, cl->act[NN_LAYERS - 1], cl->w16[NN_LAYERS - 1], cl->b32[NN_LAYERS - 1], NULL, 3, NULL, NULL,
                  cl->ugrid, gf, cl->P, 0.f);
  mgp_tstop(c, T_NNCONV);
  if (rc == MGP_OK && cufftSetStream(cl->plan_r2c, c->stream) != CUFFT_SUCCESS)
    rc = mgp_set_error(MGP_ECUFFT, "closure transform stream");
  for (int q = 0; q < 3 && rc == MGP_OK; q++)
    if (cufftExecR2C(cl->plan_r2c, (cufftReal *)(cl->ugrid + q * gf), (cufftComplex *)(cl->ugrid + q * gf)) !=
        CUFFT_SUCCESS)
      rc = mgp_set_error(MGP_ECUFFT, "closure output transform");
  if (rc == MGP_OK) {
    k_highpass<<<mgp_blocks_for(gf / 2, 4), 256, 0, c->stream>>>((float2 *)cl->ugrid, gf / 2, cl->N, cl->hp_lambda,
                                                                (float)(closure_scale(cl, A) / (double)cl->V),
                                                                (float2 *)c->frc);
    if (cudaGetLastError() != cudaSuccess) rc = mgp_set_error(MGP_ECUDA, "closure force add");
    g_kernel_launches++;
  }
  if (cl->have_plans) cufftSetStream(cl->plan_r2c, keep);
  cl->stream = keep;
  return rc;
}

// Cutoff wavelength (cells) of the sharp high-pass applied to the closure's
// output: modes of wavelength >= lambda carry no learned force (default 0:
// only the mean is removed).  A smooth filter that merely attenuates long
// waves lets the network keep large-scale output that the particle loss
// hardly sees but the dynamics integrate; a sharp one removes it, though the
// correction still reaches large scales through its coupling to the density
// (measured: lambda = 32 cells cost 0.5-1.5% of P(k) at k < 0.2 h/Mpc on the
// 256^3 workload, so the default leaves the long waves in).
extern "C" int mgp_closure_set_highpass(mgp_closure *cl, double lambda_cells) {
  if (!cl || !(lambda_cells >= 0.0)) return mgp_set_error(MGP_EINVAL, "bad closure high-pass wavelength");
  MGP_CUDA(cudaStreamSynchronize(cl->stream));
  cl->hp_lambda = (float)lambda_cells;
  return MGP_OK;
}

extern "C" double mgp_closure_get_highpass(mgp_closure *cl) { return cl ? (double)cl->hp_lambda : -1.0; }

// Residual scale s(a) used in the step (n points, a increasing, s > 0;
// n = 0 clears the table and out_scale is used).
extern "C" int mgp_closure_set_scale_table(mgp_closure *cl, int n, const double *a, const double *s) {
  if (!cl || n < 0 || (n > 0 && (!a || !s))) return mgp_set_error(MGP_EINVAL, "bad closure scale table");
  for (int q = 0; q < n; q++)
    if (!(a[q] > 0.0 && s[q] > 0.0) || (q > 0 && !(a[q] > a[q - 1])))
      return mgp_set_error(MGP_EINVAL, "closure scale table needs increasing a > 0 and s > 0");
  free(cl->scale_a);
  free(cl->scale_s);
  cl->scale_a = cl->scale_s = NULL;
  cl->scale_n = 0;
  if (n == 0) return MGP_OK;
  cl->scale_a = (double *)malloc(sizeof(double) * n);
  cl->scale_s = (double *)malloc(sizeof(double) * n);
  if (!cl->scale_a || !cl->scale_s) return mgp_set_error(MGP_ENOMEM, "closure scale table");
  memcpy(cl->scale_a, a, sizeof(double) * n);
  memcpy(cl->scale_s, s, sizeof(double) * n);
  cl->scale_n = n;
  return MGP_OK;
}

// The scale the step uses at scale factor A.
extern "C" double mgp_closure_scale_at(mgp_closure *cl, double A) { return cl ? closure_scale(cl, A) : -1.0; }

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
