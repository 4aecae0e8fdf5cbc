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
// accumulation is FP32 on the tensor cores.
//
// Layout: activations channel-last [V][16] bf16 with voxel v = (i N + j) N + k
// (k fastest, as the mesh rows); weights [27 taps][16 out][16 in], tap =
// 9 (di+1) + 3 (dj+1) + (dk+1) for offsets d in {-1, 0, 1}.
//
// Convolution as implicit GEMM on tcgen05 (k_conv_fwd_tc): per 128-voxel
// segment of an output row, 27 MMAs (M = 128 voxels, N = 16, K = 16) whose A
// operand is a staged input row shifted by dk, accumulated in tensor memory.
// The data gradient is the same convolution with the weights mirrored
// (tap -> 26 - tap) and transposed (in <-> out).  The weight gradient is,
// per tap, dY^T X over all voxels (M = N = 16 per tap, too small for the
// 128-row tcgen05 MMA): persistent blocks accumulate it in registers with
// mma.sync m16n8k16 and reduce it with one FP32 atomic per weight per block.
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
  long long own_np;                        // capacity of pc / pt
  float *pc, *pt;
  const float *cur_pc, *cur_pt;
  float *dout;                             // d loss / d out [V][4] (particle loss)
  float *fscr;                             // band-limited fine force, 3 fine grids (lazy)
  long long fscr_floats;
  // stored training samples: features (3 bf16) per voxel and either grid
  // targets (3 f32 per voxel, ds_np = 0) or particle samples (ds_np > 0)
  int nsamples, cap_samples;
  long long ds_np;
  bf16 *ds_x;
  float *ds_t, *ds_pc, *ds_pt;
};

namespace {

constexpr int kThreadsWg = 256;

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
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

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(smem_u32(smem)), "l"(gmem) : "memory");
}

// ------------------------------------------------- tcgen05 convolution
// The same convolution on the 5th-generation tensor cores: per output row
// segment of 128 voxels, D[128 x 16] (FP32, in tensor memory) accumulates 27
// MMAs (M = 128 voxels, N = 16 output channels, K = 16 input channels), one
// per tap, whose A operand is the staged input row (i+di, j+dj) shifted by dk
// voxels and whose B operand is the tap's weights, both read from shared
// memory through matrix descriptors.  A persistent CTA (one per SM) takes
// tiles of TC_I x TC_J output rows (8 accumulators, 128 TMEM columns) and
// stages the (TC_I+2) x (TC_J+2) input rows around a tile once.  Staging
// buffers and accumulators are double-buffered: while the 216 MMAs of tile t
// run (warp w issues the 27 of output row w; the eight warps'
// tcgen05.commit arrivals complete an mbarrier), the
// CTA's cp.async copies bring in tile t+1 and every warp reads its 32 TMEM
// lanes of 4 accumulators of tile t-1 (tcgen05.ld) for the epilogue.
// Shared layout (no swizzle, K-major core matrices of 8 rows x 16 bytes):
//   staged row r: [half h][voxel q][8 channels], half planes TC_Q*16 bytes
//     apart (leading byte offset), 8-voxel groups 128 bytes apart (stride
//     byte offset); a dk shift moves the start address by 16 dk bytes.
//   weights: [tap][half][out 16][8 in], 512 bytes per tap.
constexpr int TC_I = 2, TC_J = 4, TC_M = 128;
constexpr int TC_OUT = TC_I * TC_J;               // accumulators per tile
constexpr int TC_ROWS = (TC_I + 2) * (TC_J + 2);  // staged rows
constexpr int TC_Q = TC_M + 2;                    // staged voxels per row
constexpr uint32_t TC_HALF_BYTES = TC_Q * 16;
constexpr uint32_t TC_ROW_BYTES = 2 * TC_HALF_BYTES;
constexpr uint32_t TC_W_BYTES = NN_TAPS * 512;
constexpr uint32_t TC_BUF_BYTES = TC_ROWS * TC_ROW_BYTES;  // one staging buffer
constexpr uint32_t TC_TMEM_COLS = 2 * TC_OUT * 16;          // two accumulator sets
constexpr int kThreadsTc = 32 * TC_OUT;  // warp w issues and owns output row w
constexpr size_t kTcSmem = TC_W_BYTES + 2 * (size_t)TC_BUF_BYTES + 64;  // + 2 mbarriers, TMEM address
// kind::f16 instruction descriptor: D f32 (bits 4-5 = 1), A and B bf16
// (bits 7-9, 10-12 = 1), both K-major, N >> 3 at bit 17, M >> 4 at bit 24
constexpr uint32_t kTcIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((16u >> 3) << 17) | ((uint32_t)(TC_M >> 4) << 24);

__device__ int g_conv_err;  // set when a tensor-core wait gave up

// Shared-memory matrix descriptor: start, leading and stride byte offsets
// (>> 4), bits 46-48 = 0b001, base offset 0, no swizzle.
__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}
__device__ __forceinline__ void umma_bf16(uint32_t tmem_d, uint64_t da, uint64_t db, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
      "l"(da), "l"(db), "r"(idesc), "r"(acc));
}
__device__ __forceinline__ void umma_commit(uint32_t mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(mbar)
               : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }
__device__ __forceinline__ void mbar_init(uint32_t mbar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(mbar), "r"(count) : "memory");
}
// Wait for the mbarrier phase with the given parity; gives up after about
// 2e9 SM clocks (1-2 s) and returns false.
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity) {
  const long long t0 = clock64();
  for (;;) {
    uint32_t done;
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(mbar), "r"(parity)
        : "memory");
    if (done) return true;
    if (clock64() - t0 > 2000000000LL) return false;
  }
}
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
      "tcgen05.wait::ld.sync.aligned;\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int q = 0; q < 16; q++) v[q] = __uint_as_float(r[q]);
}

// Stage the input rows of tile t into a buffer (cp.async, not waited for).
__device__ __forceinline__ void tc_stage(const bf16 *__restrict__ X, int N, long long t, int nseg, int tiles_j,
                                         unsigned char *buf, int tid) {
  const int seg = (int)(t % nseg);
  const long long rest = t / nseg;
  const int i0 = (int)(rest / tiles_j) * TC_I, j0 = (int)(rest % tiles_j) * TC_J, k0 = seg * TC_M;
  const int qmax = min(TC_M + 1, N - k0 + 1);  // staged voxels past qmax are zero
  for (int c = tid; c < TC_ROWS * TC_Q * 2; c += kThreadsTc) {
    const int r = c / (TC_Q * 2), rem = c - r * (TC_Q * 2), q = rem >> 1, h = rem & 1;
    unsigned char *dst = buf + r * TC_ROW_BYTES + h * TC_HALF_BYTES + q * 16;
    if (q > qmax) {
      *reinterpret_cast<uint4 *>(dst) = make_uint4(0, 0, 0, 0);
      continue;
    }
    int ii = i0 + r / (TC_J + 2) - 1, jj = j0 + r % (TC_J + 2) - 1, kk = k0 - 1 + q;
    ii += ii < 0 ? N : 0;
    ii -= ii >= N ? N : 0;
    jj += jj < 0 ? N : 0;
    jj -= jj >= N ? N : 0;
    kk += kk < 0 ? N : 0;
    kk -= kk >= N ? N : 0;
    cp_async16(dst, X + (((long long)ii * N + jj) * N + kk) * NN_CH + 8 * h);
  }
  asm volatile("cp.async.commit_group;\n" ::: "memory");
}

// Epilogue of tile t from the accumulator set at TMEM column `acc`.
__device__ __forceinline__ void tc_epilogue(long long t, int nseg, int tiles_j, int N, int mode, uint32_t tmem_acc,
                                            int warp, int lane, const float (&bb)[16], bf16 *__restrict__ Y16,
                                            float *__restrict__ Y32, float *__restrict__ frc, long long gstride,
                                            long long P, float scale) {
  const int seg = (int)(t % nseg);
  const long long rest = t / nseg;
  const int i0 = (int)(rest / tiles_j) * TC_I, j0 = (int)(rest % tiles_j) * TC_J, k0 = seg * TC_M;
  const int lq = warp & 3, obase = (warp >> 2) * 4;  // TMEM lane quarter and 4 accumulators of this warp
  const int kk = k0 + 32 * lq + lane;
  for (int o4 = 0; o4 < 4; o4++) {
    const int o = obase + o4;
    float v[16];
    tmem_ld16(tmem_acc + ((uint32_t)(32 * lq) << 16) + o * 16, v);
    if (kk >= N) continue;
    const int i = i0 + o / TC_J, j = j0 + o % TC_J;
    const long long vx = ((long long)i * N + j) * N + kk;
#pragma unroll
    for (int q = 0; q < 16; q++) v[q] += bb[q];
    if (mode <= 1) {
      __align__(16) __nv_bfloat162 pk[8];
#pragma unroll
      for (int q = 0; q < 8; q++) {
        float a = v[2 * q], b = v[2 * q + 1];
        if (mode == 0) {
          a = fmaxf(a, 0.f);
          b = fmaxf(b, 0.f);
        }
        pk[q] = __floats2bfloat162_rn(a, b);
      }
      reinterpret_cast<uint4 *>(Y16 + vx * NN_CH)[0] = reinterpret_cast<uint4 *>(pk)[0];
      reinterpret_cast<uint4 *>(Y16 + vx * NN_CH)[1] = reinterpret_cast<uint4 *>(pk)[1];
    } else if (mode == 2) {
      reinterpret_cast<float4 *>(Y32)[vx] = make_float4(v[0], v[1], v[2], v[3]);
    } else {
      const long long gi = ((long long)i * N + j) * P + kk;
      frc[gi] += scale * v[0];
      frc[gstride + gi] += scale * v[1];
      frc[2 * gstride + gi] += scale * v[2];
    }
  }
}

__global__ void __launch_bounds__(kThreadsTc, 1) k_conv_fwd_tc(const bf16 *__restrict__ X, const bf16 *__restrict__ W,
                                                               const float *__restrict__ bias, int N, int mode,
                                                               bf16 *__restrict__ Y16, float *__restrict__ Y32,
                                                               float *__restrict__ frc, long long gstride, long long P,
                                                               float scale) {
  extern __shared__ __align__(128) unsigned char tc_smem[];
  unsigned char *ws = tc_smem;
  unsigned char *xs = tc_smem + TC_W_BYTES;  // two staging buffers
  uint64_t *mbar = reinterpret_cast<uint64_t *>(xs + 2 * (size_t)TC_BUF_BYTES);
  uint32_t *tslot = reinterpret_cast<uint32_t *>(mbar + 2);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t ws_a = smem_u32(ws), xs_a = smem_u32(xs);
  const uint32_t mbar0 = smem_u32(mbar);  // mbarrier of set b at mbar0 + 8 b
  for (int c = tid; c < NN_WSIZE / 8; c += kThreadsTc) {
    const int tap = c >> 5, o = (c >> 1) & 15, h = c & 1;
    cp_async16(ws + tap * 512 + h * 256 + o * 16, W + (size_t)c * 8);
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(tslot)),
                 "r"(TC_TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
  }
  if (tid == 0) {
    mbar_init(mbar0, TC_OUT);  // one tcgen05.commit per issuing warp
    mbar_init(mbar0 + 8, TC_OUT);
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tslot;
  const int nseg = (N + TC_M - 1) / TC_M, tiles_j = N / TC_J;
  const long long ntiles = (long long)(N / TC_I) * tiles_j * nseg;
  float bb[16];
#pragma unroll
  for (int q = 0; q < 16; q++) bb[q] = (mode != 1 && bias) ? bias[q] : 0.f;
  uint32_t ph = 0u;  // bit b: phase parity of mbarrier b
  long long prev = -1;
  int it = 0;
  bool ok = true;
  if ((long long)blockIdx.x < ntiles) tc_stage(X, N, blockIdx.x, nseg, tiles_j, xs, tid);
  for (long long t = blockIdx.x; t < ntiles; t += gridDim.x, it++) {
    const int b = it & 1;
    asm volatile("cp.async.wait_all;\n" ::: "memory");
    fence_proxy_async();  // staged rows (and weights) visible to the tensor cores
    tc_fence_before();    // TMEM reads of earlier epilogues ordered before the barrier
    __syncthreads();
    if (lane == 0) {  // warp w issues the 27 MMAs of output row w (accumulator w of set b)
      tc_fence_after();
      const int wi = warp / TC_J, wj = warp % TC_J;
      // descriptors of tap 0; a tap adds its byte offset >> 4 to the start-address field
      const uint64_t da0 = umma_desc(xs_a + b * TC_BUF_BYTES + (wi * (TC_J + 2) + wj) * TC_ROW_BYTES, TC_HALF_BYTES, 128);
      const uint64_t db0 = umma_desc(ws_a, 256, 128);
      const uint32_t d = tmem + b * (TC_OUT * 16) + warp * 16;
#pragma unroll
      for (int tap = 0; tap < NN_TAPS; tap++) {
        const int di = tap / 9, dj = (tap / 3) % 3, dk = tap % 3;
        const uint32_t offa = ((di * (TC_J + 2) + dj) * TC_ROW_BYTES + dk * 16) >> 4;
        umma_bf16(d, da0 + offa, db0 + (uint32_t)(tap * 32), kTcIdesc, tap > 0 ? 1u : 0u);
      }
      umma_commit(mbar0 + 8 * b);
    }
    if (prev >= 0) {  // tile prev: its MMAs done -> buffer b^1 free, accumulators b^1 ready
      ok = mbar_wait(mbar0 + 8 * (b ^ 1), (ph >> (b ^ 1)) & 1u);
      if (!__syncthreads_and(ok)) break;
      ph ^= 1u << (b ^ 1);
      tc_fence_after();
    }
    const long long next = t + gridDim.x;
    if (next < ntiles) tc_stage(X, N, next, nseg, tiles_j, xs + (b ^ 1) * TC_BUF_BYTES, tid);
    if (prev >= 0)
      tc_epilogue(prev, nseg, tiles_j, N, mode, tmem + (b ^ 1) * (TC_OUT * 16), warp, lane, bb, Y16, Y32, frc, gstride,
                  P, scale);
    prev = t;
  }
  if (ok && prev >= 0) {
    const int b = (it - 1) & 1;
    ok = mbar_wait(mbar0 + 8 * b, (ph >> b) & 1u);
    if (__syncthreads_and(ok)) {
      tc_fence_after();
      tc_epilogue(prev, nseg, tiles_j, N, mode, tmem + b * (TC_OUT * 16), warp, lane, bb, Y16, Y32, frc, gstride, P,
                  scale);
    }
  }
  if (!ok && tid == 0) atomicExch(&g_conv_err, 1);
  asm volatile("cp.async.wait_all;\n" ::: "memory");
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(TC_TMEM_COLS) : "memory");
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
// u_p the CIC interpolation of the network output (out [V][4], channels 0-2)
// at the particle; its gradient d loss / d out is the CIC deposit of
// 2 s (s u_p - r_p) / (3 np), accumulated into dout [V][4] (float4 atomics).
constexpr int kThreadsPl = 256;
__global__ void __launch_bounds__(kThreadsPl) k_particle_loss(const float *__restrict__ out, int N, long long np,
                                                              const float *__restrict__ pc,
                                                              const float *__restrict__ pt, float s, float inv,
                                                              float *__restrict__ dout, double *__restrict__ loss) {
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
    long long v[8];
    float wt[8];
#pragma unroll
    for (int c = 0; c < 8; c++) {
      const int bx = c >> 2, by = (c >> 1) & 1, bz = c & 1;
      v[c] = ((long long)(bx ? i1[0] : i0[0]) * N + (by ? i1[1] : i0[1])) * N + (bz ? i1[2] : i0[2]);
      wt[c] = (bx ? d[0] : 1.f - d[0]) * (by ? d[1] : 1.f - d[1]) * (bz ? d[2] : 1.f - d[2]);
    }
    float u0 = 0.f, u1 = 0.f, u2 = 0.f;
#pragma unroll
    for (int c = 0; c < 8; c++) {
      const float4 o = __ldg(reinterpret_cast<const float4 *>(out) + v[c]);
      u0 = fmaf(wt[c], o.x, u0);
      u1 = fmaf(wt[c], o.y, u1);
      u2 = fmaf(wt[c], o.z, u2);
    }
    const float e0 = s * u0 - pt[p], e1 = s * u1 - pt[np + p], e2 = s * u2 - pt[2 * np + p];
    acc += (double)e0 * e0 + (double)e1 * e1 + (double)e2 * e2;
    const float g = 2.f * s * inv;
#pragma unroll
    for (int c = 0; c < 8; c++) {
      const float gw = g * wt[c];
      atomicAdd(reinterpret_cast<float4 *>(dout) + v[c], make_float4(gw * e0, gw * e1, gw * e2, 0.f));
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

// dout [V][4] f32 -> the BF16 gradient [V][16] of the last layer (channels 0-2)
__global__ void k_dout_to_bf16(const float *__restrict__ dout, long long V, bf16 *__restrict__ g) {
  long long stride = (long long)gridDim.x * blockDim.x;
  for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < V; v += stride) {
    const float4 d = reinterpret_cast<const float4 *>(dout)[v];
    __align__(16) bf16 row[NN_CH];
#pragma unroll
    for (int c = 0; c < NN_CH; c++) row[c] = __float2bfloat16_rn(0.f);
    row[0] = __float2bfloat16_rn(d.x);
    row[1] = __float2bfloat16_rn(d.y);
    row[2] = __float2bfloat16_rn(d.z);
    reinterpret_cast<uint4 *>(g + v * NN_CH)[0] = reinterpret_cast<uint4 *>(row)[0];
    reinterpret_cast<uint4 *>(g + v * NN_CH)[1] = reinterpret_cast<uint4 *>(row)[1];
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

static int conv_fwd(mgp_closure *cl, const bf16 *X, const bf16 *W, const float *bias, int mode, bf16 *Y16, float *Y32,
                    float *frc, long long gstride, long long P, float scale) {
  static int grid = 0;  // resident CTAs of the persistent kernel (one device per process)
  if (!grid) {
    MGP_CUDA(cudaFuncSetAttribute(k_conv_fwd_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTcSmem));
    int sms = 0;
    MGP_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, cl->device));
    grid = sms;  // one CTA per SM: 213 KB of shared memory, 256 TMEM columns
  }
  const int N = cl->N;
  const long long tiles = (long long)(N / TC_I) * (N / TC_J) * ((N + TC_M - 1) / TC_M);
  const unsigned blocks = (unsigned)(tiles < grid ? tiles : grid);
  k_conv_fwd_tc<<<blocks, kThreadsTc, kTcSmem, cl->stream>>>(X, W, bias, N, mode, Y16, Y32, frc, gstride, P, scale);
  MGP_CHECK_LAUNCH();
  g_kernel_launches++;
  return MGP_OK;
}

// Error flag of the tensor-core waits (read after a synchronisation).
static int conv_status() {
  int e = 0;
  MGP_CUDA(cudaMemcpyFromSymbol(&e, g_conv_err, sizeof(int)));
  if (e) return mgp_set_error(MGP_ECUDA, "closure convolution: tensor-core completion wait timed out");
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
  if (cl->pmode) {
    MGP_CUDA(cudaMemsetAsync(cl->dout, 0, sizeof(float) * 4 * V, cl->stream));
    k_particle_loss<<<mgp_blocks_for(cl->np, 8), kThreadsPl, 0, cl->stream>>>(
        cl->out, cl->N, cl->np, cl->cur_pc, cl->cur_pt, cl->out_scale, (float)(1.0 / (3.0 * (double)cl->np)), cl->dout,
        cl->loss);
    MGP_CHECK_LAUNCH();
    k_dout_to_bf16<<<mgp_blocks_for(V, 4), 256, 0, cl->stream>>>(cl->dout, V, cl->g0);
    MGP_CHECK_LAUNCH();
    g_kernel_launches += 2;
  } else {
    k_loss_grad<<<mgp_blocks_for(V, 4), 256, 0, cl->stream>>>(cl->out, cl->target, V, cl->out_scale, cl->g0, cl->loss);
    MGP_CHECK_LAUNCH();
    g_kernel_launches++;
  }
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
  void *b[] = {cl->wt16, cl->out,  cl->target, cl->g0,   cl->g1,   cl->loss,  cl->grid_a, cl->grid_b,
               cl->ds_x, cl->ds_t, cl->ds_pc,  cl->ds_pt, cl->pc,   cl->pt,    cl->dout, cl->fscr};
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
  {
    const int zero = 0;
    CL_TRY(cudaMemcpyToSymbol(g_conv_err, &zero, sizeof(int)));
  }
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
    cl->pmode = 0;
  }
  return MGP_OK;
}

// Forward pass on the working features; out [V][3] host (may be NULL).
extern "C" int mgp_closure_forward(mgp_closure *cl, float *out) {
  if (!cl) return mgp_set_error(MGP_EINVAL, "null closure");
  MGP_CUDA(cudaSetDevice(cl->device));
  NN_RET(closure_forward(cl));
  MGP_CUDA(cudaStreamSynchronize(cl->stream));
  NN_RET(conv_status());
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
  NN_RET(conv_status());
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
    NN_RET(conv_status());
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
  if (!cl->dout) MGP_CUDA(cudaMalloc(&cl->dout, sizeof(float) * 4 * cl->V));
  return MGP_OK;
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
  if (rms) {
    MGP_CUDA(cudaMemsetAsync(cl->loss, 0, sizeof(double), cl->stream));
    k_sumsq_flat<<<mgp_blocks_for(3 * cl->np, 4), 256, 0, cl->stream>>>(cl->pt, 3 * cl->np, cl->loss);
    MGP_CHECK_LAUNCH();
    double ss = 0.0;
    MGP_CUDA(cudaMemcpyAsync(&ss, cl->loss, sizeof(double), cudaMemcpyDeviceToHost, cl->stream));
    MGP_CUDA(cudaStreamSynchronize(cl->stream));
    *rms = sqrt(ss / (3.0 * (double)cl->np));
  }
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
  if (cl->pmode && cl->cur_pc != cl->pc) cl->pmode = 0;  // the working sample pointed into the old set
  if (n == 0) return MGP_OK;
  MGP_CUDA(cudaMalloc(&cl->ds_x, sizeof(bf16) * 3 * cl->V * n));
  if (np > 0) {
    MGP_CUDA(cudaMalloc(&cl->ds_pc, sizeof(float) * 3 * np * n));
    MGP_CUDA(cudaMalloc(&cl->ds_pt, sizeof(float) * 3 * np * n));
  } else {
    MGP_CUDA(cudaMalloc(&cl->ds_t, sizeof(float) * 3 * cl->V * n));
  }
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
    if (!cl->dout) MGP_CUDA(cudaMalloc(&cl->dout, sizeof(float) * 4 * cl->V));
    const size_t n3 = (size_t)3 * cl->ds_np;
    cl->np = cl->ds_np;
    cl->cur_pc = cl->ds_pc + slot * n3;
    cl->cur_pt = cl->ds_pt + slot * n3;
    cl->pmode = 1;
  } else {
    cl->pmode = 0;
  }
  return MGP_OK;
}

// Inference inside a PM step (called by mgp_get_displacements after the
// force grids): features, three hidden layers and the last layer added to the
// force grids, on the context's stream.
int mgp_closure_apply(mgp_closure *cl, mgp_ctx *c, double A) {
  cudaStream_t keep = cl->stream;
  cl->stream = c->stream;
  int rc = closure_features(cl, c, A);
  if (c->timing) cudaEventRecord(c->ev[T_NNCONV][0], c->stream);  // the four convolutions
  for (int l = 0; l < NN_LAYERS - 1 && rc == MGP_OK; l++)
    rc = conv_fwd(cl, cl->act[l], cl->w16[l], cl->b32[l], 0, cl->act[l + 1], NULL, NULL, 0, 0, 0.f);
  if (rc == MGP_OK)
    rc = conv_fwd(cl, cl->act[NN_LAYERS - 1], cl->w16[NN_LAYERS - 1], cl->b32[NN_LAYERS - 1], 3, NULL, NULL, c->frc,
                  c->g.nreal, c->g.P, cl->out_scale);
  if (c->timing) {
    cudaEventRecord(c->ev[T_NNCONV][1], c->stream);
    c->timed[T_NNCONV] = 1;
  }
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
