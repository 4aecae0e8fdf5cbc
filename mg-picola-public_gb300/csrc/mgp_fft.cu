// The y pass of the 1024^3 half-complex transforms and the force pass fused
// into it (sm_103a).
//
// A 3D real transform of the padded [N][N][2(N/2+1)] grid is a 1D real
// transform along z over the N^2 contiguous rows and complex N-point
// transforms along y and x over the N/2+1 kz columns.  cuFFT does the z rows
// (batched 1D plans, contiguous, near the copy rate) and the x lines (a
// strided batched 1D plan); the y lines are this file's kernel, for N = 1024:
//
//   one block = 8 neighbouring kz columns of one x plane, 256 threads;
//   N = 32 x 32 (four-step): thread (b, i) loads the 32 points e = 32 a + b
//   of column i (a warp reads 4 rows x 64 contiguous bytes per load), does a
//   32-point DFT over a in registers, multiplies by W_1024^(b k1), exchanges
//   through shared memory, and thread (k1, i) does the 32-point DFT over b
//   and stores X[k1 + 32 k2] (again 4 rows x 64 bytes per warp store).
//   Every column is read once and written once: 8 bytes in and out per
//   complex value, the pass's minimum.  In place: a block owns its columns.
//   (The same kernel along x, where a block's rows lie 4.2 MB apart, ran
//   well below cuFFT's x pass; along y its rows lie 4 KB apart.)
//
// The fifth-force solvers' k-space filters (the smoothing of density
// screening, the inverse Laplacian of potential screening) ride on the first
// inverse y pass of their transform, so the P(k) pass only reads delta(k);
// the Gaussian smoothing is a product of per-axis factors (one table of 1024
// values).
//
// The force pass (Forces, src/auxPM.c:437-535) rides on the inverse y pass.
// F_a(k) = i k_a g(k) S(k), g = -1/(k^2 N^3 Scale), S = delta(k) [+ the MG
// source].  Along one y line (fixed kx, kz) F_x and F_z are fixed multiples
// (k_x, k_z) of G = i g S, so one transform of G gives both and a second,
// of k_y G, gives F_y: two transforms and one read of S write the three
// y-transformed force spectra, where k_forces wrote three spectra and three
// y passes read them back.  The Nyquist conventions of k_forces hold: on the
// kz = 0 and kz = N/2 planes a component whose own index is N/2 is zero, and
// F_z is zero on both planes.
//
// Unnormalised transforms with cuFFT's signs (forward exp(-2 pi i jk/N),
// inverse exp(+2 pi i jk/N)); the real-to-complex layout is cuFFT's and
// FFTW's (kz = 0..N/2 stored).
#include <cuda_runtime.h>
#include <cufft.h>
#include <math.h>
#include <string.h>

#include "mgp_device.cuh"
#include "mgp_internal.h"

#define RET_IF(x)                  \
  do {                             \
    int rc_ = (x);                 \
    if (rc_ != MGP_OK) return rc_; \
  } while (0)

namespace {

constexpr int FN = 1024;             // transform length
constexpr int FW = 8;                // columns per block
constexpr int FT = 256;              // threads per block: 32 rows x 8 columns
constexpr int FGR = (FN / 2) / FW;   // regular column groups (kz 0..511) per line
constexpr int FRS = 32 * FW + 8;     // shared-memory row of one k1 (float2), padded
constexpr int FSMEM = 32 * FRS * 8;  // bytes of the exchange buffer
constexpr int FBLOCKS = FN * FGR + FN / FW;  // regular groups + Nyquist-column groups

enum { PASS_PLAIN = 0, PASS_FORCE = 1, PASS_FILTER = 2 };

__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cmul(float2 a, float2 w) {
  return make_float2(fmaf(a.x, w.x, -a.y * w.y), fmaf(a.x, w.y, a.y * w.x));
}
__device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }

// cos(2 pi m / 32) for m = 0..8 (the decimal expansions of the exact values)
__device__ __forceinline__ float cos32(int m) {
  switch (m) {
    case 0: return 1.0f;
    case 1: return 0.98078528040323044913f;
    case 2: return 0.92387953251128675613f;
    case 3: return 0.83146961230254523708f;
    case 4: return 0.70710678118654752440f;
    case 5: return 0.55557023301960222474f;
    case 6: return 0.38268343236508977173f;
    case 7: return 0.19509032201612826785f;
    default: return 0.0f;
  }
}

// d * W32^m, W32 = exp(DIR 2 pi i / 32), m = 0..15 a compile-time constant
// after unrolling (m = 0 and m = 8 without multiplications).
template <int DIR>
__device__ __forceinline__ float2 twmul(float2 d, int m) {
  if (m == 0) return d;
  if (m == 8) return DIR > 0 ? make_float2(-d.y, d.x) : make_float2(d.y, -d.x);
  const float c = m <= 8 ? cos32(m) : -cos32(16 - m);
  const float s = m <= 8 ? cos32(8 - m) : cos32(m - 8);
  return cmul(d, make_float2(c, DIR > 0 ? s : -s));
}

// 32-point DFT in registers, radix-2 decimation in frequency: natural-order
// input, output X[k] in v[bitrev5(k)].
template <int DIR>
__device__ __forceinline__ void dft32(float2 (&v)[32]) {
#pragma unroll
  for (int h = 16; h >= 1; h >>= 1) {
#pragma unroll
    for (int s = 0; s < 32; s += 2 * h) {
#pragma unroll
      for (int j = 0; j < h; j++) {
        const float2 a = v[s + j], b = v[s + j + h];
        v[s + j] = cadd(a, b);
        v[s + j + h] = twmul<DIR>(csub(a, b), j * (16 / h));
      }
    }
  }
}

__host__ __device__ constexpr int bitrev5(int r) {
  return ((r & 1) << 4) | ((r & 2) << 2) | (r & 4) | ((r & 8) >> 2) | ((r & 16) >> 4);
}

// Signed wave number of a stored index (N/2 stays +N/2).
__device__ __forceinline__ int wave(int i) { return i > FN / 2 ? i - FN : i; }

// The four-step transform of the block's 8 columns held as v[a] = x[32 a + b]
// (thread t: b = t / 8, column t % 8); on return v[r] = X[k1 + 32 bitrev5(r)]
// with k1 = t / 8.  tw = W_1024^m, m = 0..1023, forward sign.
template <int DIR>
__device__ __forceinline__ void four_step(float2 (&v)[32], float2 *S, const float2 *__restrict__ tw) {
  const int t = threadIdx.x, i = t & 7, b = t >> 3;
  // W_1024^(b k1) = W^(b (k1 & 7)) W^(b (k1 & 24)): 12 table entries per
  // thread instead of 32 (the product of two rounded entries, ~1 ulp more)
  dft32<DIR>(v);
  float2 t1[8], t2[4];
#pragma unroll
  for (int l = 0; l < 8; l++) t1[l] = __ldg(tw + b * l);
#pragma unroll
  for (int m = 0; m < 4; m++) t2[m] = __ldg(tw + 8 * b * m);
  // v[r] = Y[b][k1], k1 = bitrev5(r): twiddle W_1024^(b k1), to S[k1][b][i]
#pragma unroll
  for (int r = 0; r < 32; r++) {
    const int k1 = bitrev5(r), lo = k1 & 7, hi = k1 >> 3;
    float2 w = lo == 0 ? t2[hi] : (hi == 0 ? t1[lo] : cmul(t1[lo], t2[hi]));
    if (DIR > 0) w.y = -w.y;
    S[k1 * FRS + b * FW + i] = k1 == 0 ? v[r] : cmul(v[r], w);
  }
  __syncthreads();
#pragma unroll
  for (int bb = 0; bb < 32; bb++) v[bb] = S[b * FRS + bb * FW + i];  // thread (k1 = b, i)
  dft32<DIR>(v);
}

// Columns of the block: regular groups are kz0..kz0+7 of one line `outer`;
// the last FN/8 blocks take the Nyquist column kz = N/2 of 8 lines.
__device__ __forceinline__ void block_column(int blk, int i, unsigned os, int &outer, int &kz, unsigned &base) {
  if (blk < FN * FGR) {
    outer = blk / FGR;
    kz = (blk - outer * FGR) * FW + i;
  } else {
    outer = (blk - FN * FGR) * FW + i;
    kz = FN / 2;
  }
  base = (unsigned)outer * os + (unsigned)kz;
}

// Store v[r] = X[k1 + 32 bitrev5(r)] (k1 = t / 8) times `mult`.
__device__ __forceinline__ void store_column(const float2 (&v)[32], float2 *out, unsigned base, unsigned es,
                                             float mult, bool scaled) {
  const int b = threadIdx.x >> 3;
#pragma unroll
  for (int r = 0; r < 32; r++) out[base + (unsigned)(b + 32 * bitrev5(r)) * es] = scaled ? cscale(v[r], mult) : v[r];
}

// The y pass over a half-complex N^3 grid: element e (the y index) of
// column (x = outer, kz) at outer*N*NH + e*NH + kz (float2 units).
//   PASS_PLAIN: out = DFT(in) (out may be in: a block owns its columns)
//   PASS_FORCE: inverse y pass of the forces from in = S: two blocks per
//               column group, adjacent in launch order so that the second
//               one's read of S finds it in L2 (one transform per block
//               keeps the kernel within 128 registers).  Phase 0: T =
//               transform of G = i g S, g = cfac/k^2; fx = k_x T, fz = k_z T.
//               Phase 1: fy = transform of k_y G.  None of fx, fy, fz is in.
//   PASS_FILTER: out = DFT(f(|k|^2) in), f = mg_kfilter (the smoothing or
//               inverse-Laplacian filter of the fifth-force solvers); out is
//               not in.
struct yfilter {
  int kind, filter;  // mg_kfilter's
  float kR1, norm;
  const float *gauss;  // Gaussian smoothing: exp(-(kR1 d)^2 / 2) per stored index (d its wave number), or NULL
};

template <int DIR, int MODE>
__global__ void __launch_bounds__(FT, 2) k_fft_y(const float2 *in, float2 *out, float2 *fx, float2 *fy, float2 *fz,
                                                 const float2 *__restrict__ tw, float cfac, yfilter yf) {
  extern __shared__ __align__(16) float2 S[];
  constexpr unsigned NH = FN / 2 + 1, OS = FN * NH, ES = NH;
  const int t = threadIdx.x, i = t & 7, b = t >> 3;
  const int group = MODE == PASS_FORCE ? (int)(blockIdx.x >> 1) : (int)blockIdx.x;
  const int phase = MODE == PASS_FORCE ? (int)(blockIdx.x & 1) : 0;
  int outer, kz;
  unsigned base;
  block_column(group, i, OS, outer, kz, base);
  float2 v[32];
  if (MODE == PASS_PLAIN) {
#pragma unroll
    for (int a = 0; a < 32; a++) v[a] = in[base + (unsigned)(32 * a + b) * ES];
    four_step<DIR>(v, S, tw);
    store_column(v, out, base, ES, 1.0f, false);
    return;
  }
  if (MODE == PASS_FILTER) {
    const int dx = wave(outer), r0 = dx * dx + kz * kz;
#pragma unroll
    for (int a = 0; a < 32; a++) v[a] = in[base + (unsigned)(32 * a + b) * ES];
    if (yf.gauss) {
      // the Gaussian is a product over the axes: norm G(kx) G(kz) per column
      // times G(ky) per element
      const float gxz = yf.norm * __ldg(yf.gauss + outer) * __ldg(yf.gauss + kz);
#pragma unroll
      for (int a = 0; a < 32; a++) v[a] = cscale(v[a], gxz * __ldg(yf.gauss + 32 * a + b));
    } else {
#pragma unroll
      for (int a = 0; a < 32; a++) {
        const int dy = wave(32 * a + b);
        v[a] = cscale(v[a], mg_kfilter(dy * dy + r0, yf.kind, yf.filter, yf.kR1, yf.norm));
      }
    }
    four_step<DIR>(v, S, tw);
    store_column(v, out, base, ES, 1.0f, false);
    return;
  }
  const bool nyq_plane = kz == 0 || 2 * kz == FN;
  const int dx = wave(outer), r0 = dx * dx + kz * kz;
  // all 32 loads first: the division's branches would otherwise keep the
  // compiler from issuing the later loads before the earlier arithmetic
#pragma unroll
  for (int a = 0; a < 32; a++) v[a] = in[base + (unsigned)(32 * a + b) * ES];
#pragma unroll
  for (int a = 0; a < 32; a++) {
    const int e = 32 * a + b, dy = wave(e), rk = dy * dy + r0;
    float g = rk == 0 ? 0.0f : cfac / (float)rk;
    if (phase) g *= (nyq_plane && 2 * e == FN) ? 0.0f : (float)dy;
    v[a] = make_float2(-g * v[a].y, g * v[a].x);
  }
  four_step<DIR>(v, S, tw);
  if (phase) {
    store_column(v, fy, base, ES, 1.0f, false);
  } else {
    store_column(v, fx, base, ES, (nyq_plane && 2 * outer == FN) ? 0.0f : (float)dx, true);
    store_column(v, fz, base, ES, nyq_plane ? 0.0f : (float)kz, true);
  }
}

template <int DIR, int MODE>
int launch_y(const float2 *in, float2 *out, float2 *fx, float2 *fy, float2 *fz, const float2 *tw, float cfac,
             cudaStream_t st, yfilter yf = yfilter{0, 0, 0.f, 0.f, NULL}) {
  MGP_CUDA(cudaFuncSetAttribute(k_fft_y<DIR, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, FSMEM));
  k_fft_y<DIR, MODE><<<MODE == PASS_FORCE ? 2 * FBLOCKS : FBLOCKS, FT, FSMEM, st>>>(in, out, fx, fy, fz, tw, cfac,
                                                                                   yf);
  MGP_CHECK_LAUNCH();
  g_kernel_launches++;
  return MGP_OK;
}

}  // namespace

// Whether the context's grid takes the y pass of this file.
int mgp_fft_supported(const mgp_ctx *c) { return c->g.N == FN && c->nbox == 1; }

// z-direction plans (batched 1D over the N^2 rows), the strided x plan (1D
// C2C over the N NH (y, kz) columns, element stride N NH) and the twiddle
// table.
int mgp_fft_setup(mgp_ctx *c) {
  if (c->fft_ready) return MGP_OK;
  if (!mgp_fft_supported(c)) return mgp_set_error(MGP_EINVAL, "the y pass needs Nmesh = %d", FN);
  const long long N = c->g.N, P = c->g.P, NH = c->g.NH;
  long long n[1] = {N}, rembed[1] = {P}, cembed[1] = {NH}, xembed[1] = {N};
  size_t ws[4] = {0, 0, 0, 0};
  cufftHandle *plans[4] = {&c->zplan_r2c_oop, &c->zplan_r2c_ip, &c->zplan_c2r, &c->xplan};
  for (int k = 0; k < 4; k++) {
    MGP_CUFFT(cufftCreate(plans[k]));
    MGP_CUFFT(cufftSetAutoAllocation(*plans[k], 0));
  }
  MGP_CUFFT(cufftMakePlanMany64(c->zplan_r2c_oop, 1, n, rembed, 1, P, cembed, 1, NH, CUFFT_R2C, N * N, &ws[0]));
  MGP_CUFFT(cufftMakePlanMany64(c->zplan_r2c_ip, 1, n, rembed, 1, P, cembed, 1, NH, CUFFT_R2C, N * N, &ws[1]));
  MGP_CUFFT(cufftMakePlanMany64(c->zplan_c2r, 1, n, cembed, 1, NH, rembed, 1, P, CUFFT_C2R, N * N, &ws[2]));
  MGP_CUFFT(cufftMakePlanMany64(c->xplan, 1, n, xembed, N * NH, 1, xembed, N * NH, 1, CUFFT_C2C, N * NH, &ws[3]));
  size_t need = 0;
  for (int k = 0; k < 4; k++) need = ws[k] > need ? ws[k] : need;
  if (need > c->fft_work_bytes) {
    void *w = NULL;
    MGP_CUDA(cudaMalloc(&w, need));
    if (c->fft_work) cudaFree(c->fft_work);
    c->fft_work = w;
    c->fft_work_bytes = need;
    // the 3D plans share the work area
    cufftHandle p3[3] = {c->plan_r2c_oop, c->plan_r2c_ip, c->plan_c2r_1};
    for (int k = 0; k < 3; k++)
      if (p3[k]) MGP_CUFFT(cufftSetWorkArea(p3[k], c->fft_work));
  }
  for (int k = 0; k < 4; k++) {
    MGP_CUFFT(cufftSetWorkArea(*plans[k], c->fft_work));
    MGP_CUFFT(cufftSetStream(*plans[k], c->stream));
  }
  // W_1024^m = exp(-2 pi i m / 1024), evaluated in double
  float2 h[FN];
  for (int m = 0; m < FN; m++) {
    const double ang = -2.0 * M_PI * (double)m / (double)FN;
    h[m] = make_float2((float)cos(ang), (float)sin(ang));
  }
  MGP_CUDA(cudaMalloc(&c->fft_tw, sizeof(h)));
  MGP_CUDA(cudaMemcpy(c->fft_tw, h, sizeof(h), cudaMemcpyHostToDevice));
  c->fft_ready = 1;
  return MGP_OK;
}

void mgp_fft_free(mgp_ctx *c) {
  cufftHandle plans[4] = {c->zplan_r2c_oop, c->zplan_r2c_ip, c->zplan_c2r, c->xplan};
  for (int k = 0; k < 4; k++)
    if (plans[k]) cufftDestroy(plans[k]);
  c->zplan_r2c_oop = c->zplan_r2c_ip = c->zplan_c2r = c->xplan = 0;
  if (c->fft_tw) cudaFree(c->fft_tw);
  if (c->fft_gauss) cudaFree(c->fft_gauss);
  c->fft_tw = NULL;
  c->fft_gauss = NULL;
  c->fft_ready = 0;
}

// Forward real-to-complex transform of a padded real grid (in place when
// out == in): z rows, the y pass, the x lines.
int mgp_fft_r2c(mgp_ctx *c, float *in, float *out) {
  RET_IF(mgp_fft_setup(c));
  const cufftHandle pz = in == out ? c->zplan_r2c_ip : c->zplan_r2c_oop;
  MGP_CUFFT(cufftExecR2C(pz, (cufftReal *)in, (cufftComplex *)out));
  float2 *o = (float2 *)out;
  RET_IF((launch_y<-1, PASS_PLAIN>(o, o, NULL, NULL, NULL, (const float2 *)c->fft_tw, 0.f, c->stream)));
  MGP_CUFFT(cufftExecC2C(c->xplan, (cufftComplex *)out, (cufftComplex *)out, CUFFT_FORWARD));
  return MGP_OK;
}

// Inverse complex-to-real transform in place: the x lines, the y pass, the
// z rows.
int mgp_fft_c2r(mgp_ctx *c, float *grid) {
  RET_IF(mgp_fft_setup(c));
  float2 *g = (float2 *)grid;
  MGP_CUFFT(cufftExecC2C(c->xplan, (cufftComplex *)grid, (cufftComplex *)grid, CUFFT_INVERSE));
  RET_IF((launch_y<1, PASS_PLAIN>(g, g, NULL, NULL, NULL, (const float2 *)c->fft_tw, 0.f, c->stream)));
  MGP_CUFFT(cufftExecC2R(c->zplan_c2r, (cufftComplex *)grid, (cufftReal *)grid));
  return MGP_OK;
}

// Inverse transform of f(|k|^2) in(k) into `out` (in is kept): the
// smoothing (kind 1: filter, kR1, norm) or inverse-Laplacian (kind 2: norm)
// filter of the fifth-force solvers applied in the y pass, then the x lines
// and z rows of out.
int mgp_fft_c2r_filtered(mgp_ctx *c, const float *in, float *out, int kind, int filter, float kR1, float norm) {
  RET_IF(mgp_fft_setup(c));
  const float *gauss = NULL;
  if (kind == 1 && filter == MGP_FILTER_GAUSSIAN) {
    // exp(-(kR1 d)^2 / 2) per stored index, d = its wave number (FP64 on the host)
    if (!c->fft_gauss) MGP_CUDA(cudaMalloc(&c->fft_gauss, sizeof(float) * FN));
    if (c->fft_gauss_kR1 != kR1) {
      float h[FN];
      for (int i = 0; i < FN; i++) {
        const double d = i > FN / 2 ? i - FN : i, x = (double)kR1 * d;
        h[i] = (float)exp(-0.5 * x * x);
      }
      MGP_CUDA(cudaMemcpy(c->fft_gauss, h, sizeof(h), cudaMemcpyHostToDevice));
      c->fft_gauss_kR1 = kR1;
    }
    gauss = c->fft_gauss;
  }
  RET_IF((launch_y<1, PASS_FILTER>((const float2 *)in, (float2 *)out, NULL, NULL, NULL, (const float2 *)c->fft_tw,
                                   0.f, c->stream, yfilter{kind, filter, kR1, norm, gauss})));
  MGP_CUFFT(cufftExecC2C(c->xplan, (cufftComplex *)out, (cufftComplex *)out, CUFFT_INVERSE));
  MGP_CUFFT(cufftExecC2R(c->zplan_c2r, (cufftComplex *)out, (cufftReal *)out));
  return MGP_OK;
}

// The force pass and the three inverse transforms (Forces,
// src/auxPM.c:437-555) of one spectrum S(k): delta(k), or delta plus the MG
// source when the screening pass has summed them; `mult` scales S (1 +
// coupling for nDGP without screening, else 1).  The fused y pass writes
// the three y-transformed force spectra from one read of S; each force grid
// then takes its x lines and z rows.  The fused pass runs under timer t_x,
// the rest under t_rest.
int mgp_fft_forces(mgp_ctx *c, const float *spec, float mult, int t_x, int t_rest) {
  RET_IF(mgp_fft_setup(c));
  const unsigned N = (unsigned)c->g.N;
  const double scale = 2.0 * M_PI / c->p.Box;
  const float cfac = (float)(-1.0 / ((double)N * N * N * scale)) * mult;
  float *f[3] = {c->frc, c->frc + c->g.nreal, c->frc + 2 * c->g.nreal};
  mgp_tstart(c, t_x);
  RET_IF((launch_y<1, PASS_FORCE>((const float2 *)spec, NULL, (float2 *)f[0], (float2 *)f[1], (float2 *)f[2],
                                  (const float2 *)c->fft_tw, cfac, c->stream)));
  mgp_tstop(c, t_x);
  mgp_tstart(c, t_rest);
  for (int a = 0; a < 3; a++) {
    MGP_CUFFT(cufftExecC2C(c->xplan, (cufftComplex *)f[a], (cufftComplex *)f[a], CUFFT_INVERSE));
    MGP_CUFFT(cufftExecC2R(c->zplan_c2r, (cufftComplex *)f[a], (cufftReal *)f[a]));
  }
  mgp_tstop(c, t_rest);
  return MGP_OK;
}
