// CUDA kernels of the GB300 COLA particle-mesh step and 2LPT IC path
// (sm_103a).  Every kernel restates one loop of the reference and cites it;
// paths are relative to the MG-PICOLA-PUBLIC tree.
//
// All kernels are HBM-bound streaming or gather/scatter passes: none of them
// is GEMM-shaped, so there is no tensor-core path here.  Grids are sized in
// multiples of the SM count (152 on GB300) times resident blocks.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#include "mgp_device.cuh"
#include "mgp_internal.h"
#include "mgp_rng.h"

#define MGP_THREADS 256

// Process-wide count of this library's own kernel launches (cuFFT not
// included); read by mgp_launch_count.
long long g_kernel_launches = 0;
long long mgp_kernel_launches(void) { return g_kernel_launches; }

static int g_sm_count = 0;
static int sm_count() {
  if (g_sm_count == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&g_sm_count, cudaDevAttrMultiProcessorCount, dev);
    if (g_sm_count <= 0) g_sm_count = 152;
  }
  return g_sm_count;
}

static int blocks_for(long long n, int per_sm) {
  long long b = (n + MGP_THREADS - 1) / MGP_THREADS;
  long long cap = (long long)sm_count() * per_sm;
  if (b > cap) b = cap;
  if (b < 1) b = 1;
  return (int)b;
}
int mgp_blocks_for(long long n, int per_sm) { return blocks_for(n, per_sm); }
// Grid over `nbox` independent boxes: blockIdx.y is the box, and the x
// blocks of all boxes together stay near the single-box budget.
static dim3 grid_boxes(long long n_per_box, int per_sm, int nbox) {
  long long b = (n_per_box + MGP_THREADS - 1) / MGP_THREADS;
  long long cap = ((long long)sm_count() * per_sm + nbox - 1) / nbox;
  if (b > cap) b = cap;
  if (b < 1) b = 1;
  return dim3((unsigned)b, (unsigned)nbox);
}
int mgp_blocks_per_box(long long n_per_box, int per_sm, int nbox) { return (int)grid_boxes(n_per_box, per_sm, nbox).x; }

// Launch budgets (resident blocks per SM) of the deposit and of the grid
// passes.  A batch sets its tuned values while its graph is captured and
// restores these defaults afterwards.
static int g_budget_cic = MGP_BUDGET_DEFAULT, g_budget_grid = MGP_BUDGET_DEFAULT;
void mgp_set_launch_budget(int cic, int grid) {
  g_budget_cic = cic > 0 ? cic : MGP_BUDGET_DEFAULT;
  g_budget_grid = grid > 0 ? grid : MGP_BUDGET_DEFAULT;
}

// -------------------------------------------------------------- helpers
__global__ void k_fill(float *__restrict__ p, long long n, float v) {
  long long stride = (long long)gridDim.x * blockDim.x;
  long long n4 = n >> 2;  // grids are 256-byte aligned; n % 4 tail handled below
  float4 v4 = make_float4(v, v, v, v);
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += stride)
    reinterpret_cast<float4 *>(p)[i] = v4;
  for (long long i = 4 * n4 + (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) p[i] = v;
}

int mgp_launch_fill(float *p, long long n, float value, cudaStream_t st) {
  k_fill<<<blocks_for(n, g_budget_grid), MGP_THREADS, 0, st>>>(p, n, value);
  MGP_CHECK_LAUNCH();
  g_kernel_launches++;
  return MGP_OK;
}

// ------------------------------------------------------------- CIC deposit
// PtoMesh (src/auxPM.c:280-357): every particle adds its cloud-in-cell
// weights, with WPAR = (N/Ns)^3 folded into the y factors (auxPM.c:316-317),
// to a density grid pre-set to -1; periodic in all three axes (the ghost
// x-slice exchange of auxPM.c:350-356 is the x wrap).
// P2: Ns = 2^ls, lattice and cell index arithmetic by shifts (identical
// results).  IDX: offset type inside one box's grid, 32-bit when the padded
// grid has fewer than 2^31 floats (N <= 1024), which saves the 64-bit
// multiplies of the eight addresses.
template <bool P2, typename IDX>
__global__ void __launch_bounds__(MGP_THREADS) k_cic(const float *__restrict__ s, const mgp_dstate *__restrict__ st,
                                                     long long np, int Ns, int ls, int N, float scale, float wpar,
                                                     float *__restrict__ rho, long long P, long long g_bs,
                                                     long long p0, long long p1) {
  // box blockIdx.y of a batch: particles 3 np apart, grids g_bs floats apart
  s += blockIdx.y * 3 * np;
  st += blockIdx.y;
  rho += blockIdx.y * g_bs;
  const float ox = (float)(st->cx[0] * scale), oy = (float)(st->cx[1] * scale), oz = (float)(st->cx[2] * scale);
  const float inv_ns = 1.0f / (float)Ns;
  const float *sx = s, *sy = s + np, *sz = s + 2 * np;
  const IDX Pi = (IDX)P, NPi = (IDX)N * (IDX)P;
  long long stride = (long long)gridDim.x * blockDim.x;
  for (long long p = p0 + (long long)blockIdx.x * blockDim.x + threadIdx.x; p < p1; p += stride) {
    int i, j, k;
    int ix, iy, iz;
    float DX, DY, DZ;
    if (P2) {
      lattice_ijk_p2((unsigned)p, ls, i, j, k);
      cell_frac_p2(i, sx[p], ox, N, ls, inv_ns, scale, ix, DX);
      cell_frac_p2(j, sy[p], oy, N, ls, inv_ns, scale, iy, DY);
      cell_frac_p2(k, sz[p], oz, N, ls, inv_ns, scale, iz, DZ);
    } else {
      if (np <= 0xffffffffLL)
        lattice_ijk((unsigned)p, Ns, i, j, k);
      else
        lattice_ijk(p, Ns, i, j, k);
      cell_frac(i, sx[p], ox, N, Ns, scale, ix, DX);
      cell_frac(j, sy[p], oy, N, Ns, scale, iy, DY);
      cell_frac(k, sz[p], oz, N, Ns, scale, iz, DZ);
    }
    float TX = 1.0f - DX, TY = (1.0f - DY) * wpar, TZ = 1.0f - DZ;
    DY *= wpar;
    const IDX x0 = (IDX)ix * NPi, x1 = (ix + 1 == N ? 0 : (IDX)(ix + 1) * NPi);
    const IDX y0 = (IDX)iy * Pi, y1 = (iy + 1 == N ? 0 : (IDX)(iy + 1) * Pi);
    const IDX z0 = (IDX)iz, z1 = (iz + 1 == N ? 0 : (IDX)(iz + 1));
    float *r00 = rho + (x0 + y0), *r01 = rho + (x0 + y1), *r10 = rho + (x1 + y0), *r11 = rho + (x1 + y1);
    atomicAdd(r00 + z0, TX * TY * TZ);
    atomicAdd(r00 + z1, TX * TY * DZ);
    atomicAdd(r01 + z0, TX * DY * TZ);
    atomicAdd(r01 + z1, TX * DY * DZ);
    atomicAdd(r10 + z0, DX * TY * TZ);
    atomicAdd(r10 + z1, DX * TY * DZ);
    atomicAdd(r11 + z0, DX * DY * TZ);
    atomicAdd(r11 + z1, DX * DY * DZ);
  }
}

static void launch_cic(dim3 grid, const float *s, const mgp_dstate *st, long long np, int Ns, int N, double box,
                       float wpar, float *rho, long long P, long long g_bs, long long p0, long long p1,
                       cudaStream_t stream) {
  const int ls = lattice_log2(Ns);
  const bool p2 = ls >= 0 && np <= 0xffffffffLL;
  const bool i32 = (long long)N * N * P < (1LL << 31);
  const float sc = (float)(N / box);
  if (p2 && i32)
    k_cic<true, int><<<grid, MGP_THREADS, 0, stream>>>(s, st, np, Ns, ls, N, sc, wpar, rho, P, g_bs, p0, p1);
  else if (p2)
    k_cic<true, long long><<<grid, MGP_THREADS, 0, stream>>>(s, st, np, Ns, ls, N, sc, wpar, rho, P, g_bs, p0, p1);
  else if (i32)
    k_cic<false, int><<<grid, MGP_THREADS, 0, stream>>>(s, st, np, Ns, ls, N, sc, wpar, rho, P, g_bs, p0, p1);
  else
    k_cic<false, long long><<<grid, MGP_THREADS, 0, stream>>>(s, st, np, Ns, ls, N, sc, wpar, rho, P, g_bs, p0, p1);
}

int mgp_launch_cic(const float *s, const mgp_dstate *st, long long np, int Ns, int N, double box, float wpar,
                   float *rho, long long P, cudaStream_t stream, int nbox, long long g_bs) {
  launch_cic(grid_boxes(np, g_budget_cic, nbox), s, st, np, Ns, N, box, wpar, rho, P, g_bs, 0, np, stream);
  MGP_CHECK_LAUNCH();
  g_kernel_launches++;
  return MGP_OK;
}

// one box, particles p0 .. p1-1 (deposits of the chunks of a host upload)
int mgp_launch_cic_range(const float *s, const mgp_dstate *st, long long np, long long p0, long long p1, int Ns, int N,
                         double box, float wpar, float *rho, long long P, cudaStream_t stream) {
  if (p1 <= p0) return MGP_OK;
  launch_cic(grid_boxes(p1 - p0, g_budget_cic, 1), s, st, np, Ns, N, box, wpar, rho, P, 0, p0, p1, stream);
  MGP_CHECK_LAUNCH();
  g_kernel_launches++;
  return MGP_OK;
}

// ------------------------------------------------------------- P(k) bins
// compute_power_spectrum (src/compute_pofk.c:71-271): every stored mode
// (i, j, kz), kz in [0, N/2], contributes |delta|^2 / (sinc_x sinc_y sinc_z)^4
// with weight 1 on the kz = 0 and kz = N/2 planes and 2 elsewhere; the
// y-mirror loop of the reference visits exactly the stored j range.  The bin
// of a mode depends only on its integer |k|^2, looked up in rk_bin (computed
// on the host in double exactly as pofk_bin_index, compute_pofk.c:30-46).
// Mode counts and k sums are geometric and also precomputed on the host.
//
// Accumulation: a warp reads 32 consecutive modes (coalesced); lanes with the
// same bin are contiguous (|k| grows along kz), so a segmented warp scan sums
// each run in FP32 and the last lane of a run adds it to an FP64 shared-memory
// bin; blocks write FP64 partials that k_pofk_reduce sums in fixed order.
// Bin lookup: with `thr` (first |k|^2 of every bin, thr[nbins] = end of the
// binned range; bins are monotone in |k|^2) a float estimate of the bin is
// corrected against the exact integer thresholds held in shared memory, which
// reproduces the host's double-precision pofk_bin_index for every mode;
// without it the per-|k|^2 table rk_bin is read from global memory.
// Fused k-space output (one read of delta(k) serves both): fuse_kind 1 writes
// delta(k) W(kR) norm (SmoothDensityField, src/mg.h:268-309), 2 writes
// -norm delta(k)/RK (DivideByLaplacian, src/mg.h:21-64).
struct mgp_pofk_kargs {
  const float2 *dk;
  int N, nbins, bintype;
  const int *rk_bin;   // used when thr == NULL
  const int *thr;      // nbins + 1 thresholds, or NULL
  const float *win;
  float kmin, kmax;    // integer-k units (estimate only)
  double *block_part;
  int fuse_kind, filter;
  float2 *fuse_out;
  float fuse_a, fuse_b;
  int priv;
  long long dk_bs;     // box stride of dk / fuse_out (complex values)
  long long part_bs;   // box stride of block_part (doubles)
};

// Bin sums: native FP32 shared-memory atomics made exact to second order by
// a compensated (TwoSum) split: the atomic returns the old value, so the
// rounding error of every addition is recovered and added to a second FP32
// array; hi + lo carries about twice FP32's precision.
// priv != 0: every warp owns its own hi/lo bin arrays (the run tails of one
// warp always hit distinct bins), so the sums need no atomics at all.
__global__ void __launch_bounds__(MGP_THREADS) k_pofk(mgp_pofk_kargs a) {
  extern __shared__ float shf[];
  const int N = a.N, nbins = a.nbins, NH = N / 2 + 1, h = N / 2;
  const float2 *__restrict__ dkb = a.dk + blockIdx.y * a.dk_bs;
  float2 *__restrict__ fob = a.fuse_out ? a.fuse_out + blockIdx.y * a.dk_bs : nullptr;
  double *__restrict__ bpb = a.block_part + blockIdx.y * a.part_bs;
  const int nwb = a.priv ? (int)(blockDim.x >> 5) : 1;
  float *shi0 = shf, *slo0 = shf + nwb * nbins;
  int *sthr = (int *)(slo0 + nwb * nbins);
  float *swin = (float *)(sthr + (a.thr ? nbins + 1 : 0));
  for (int b = threadIdx.x; b < nwb * nbins; b += blockDim.x) shi0[b] = slo0[b] = 0.0f;
  const int wslot = a.priv ? (int)(threadIdx.x >> 5) : 0;
  float *shi = shi0 + wslot * nbins, *slo = slo0 + wslot * nbins;
  if (a.thr)
    for (int b = threadIdx.x; b <= nbins; b += blockDim.x) sthr[b] = a.thr[b];
  for (int d = threadIdx.x; d <= h; d += blockDim.x) swin[d] = a.win[d];
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const long long wid = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
  const float inv_span = (float)nbins / (a.kmax - a.kmin);
  const float inv_logspan = a.bintype ? (float)nbins / logf(a.kmax / a.kmin) : 0.0f;
  const int lo = a.thr ? sthr[0] : 0, hi = a.thr ? sthr[nbins] : 0;
  // One warp per (|d0|, |d1|) pair: the up to four stored rows (i, j) with
  // i in {d0, N-d0}, j in {d1, N-d1} share |k|^2 along kz, hence the bins,
  // window and filter; their powers are summed before the warp scan.
  const long long npair = (long long)(h + 1) * (h + 1);
  for (long long q = wid; q < npair; q += nw) {
    const int d0 = (int)(q / (h + 1)), d1 = (int)(q - (long long)d0 * (h + 1));
    const int rk01 = d0 * d0 + d1 * d1;
    const float w01 = swin[d0] * swin[d1];
    const bool mi = !(d0 == 0 || d0 == h), mj = !(d1 == 0 || d1 == h);
    const long long rows[4] = {(long long)d0 * N + d1, (long long)d0 * N + (N - d1), (long long)(N - d0) * N + d1,
                               (long long)(N - d0) * N + (N - d1)};
    const bool use[4] = {true, mj, mi, mi && mj};
    // the rows' next 32 modes are loaded while the current ones are binned
    float2 zn[4];
#pragma unroll
    for (int t = 0; t < 4; t++)
      if (use[t] && lane < NH) zn[t] = dkb[rows[t] * NH + lane];
    for (int k0 = 0; k0 < NH; k0 += 32) {
      const int kz = k0 + lane;
      float2 z[4];
#pragma unroll
      for (int t = 0; t < 4; t++) z[t] = zn[t];
      if (kz + 32 < NH) {
#pragma unroll
        for (int t = 0; t < 4; t++)
          if (use[t]) zn[t] = dkb[rows[t] * NH + kz + 32];
      }
      int bin = -1;
      float pk = 0.0f;
      if (kz < NH) {
        const int rk = rk01 + kz * kz;
        if (a.thr) {
          if (rk >= lo && rk < hi) {
            float km = sqrtf((float)rk);
            float x = a.bintype ? logf(km / a.kmin) * inv_logspan : (km - a.kmin) * inv_span;
            int b = (int)floorf(x + 0.5f);
            b = b < 0 ? 0 : (b >= nbins ? nbins - 1 : b);
            while (b > 0 && sthr[b] > rk) b--;
            while (b + 1 < nbins && sthr[b + 1] <= rk) b++;
            bin = b;
          }
        } else {
          bin = a.rk_bin[rk];
        }
        const float f = a.fuse_kind ? mg_kfilter(rk, a.fuse_kind, a.filter, a.fuse_a, a.fuse_b) : 0.0f;
        float p2 = 0.0f;
#pragma unroll
        for (int t = 0; t < 4; t++)
          if (use[t]) {
            p2 += z[t].x * z[t].x + z[t].y * z[t].y;
            if (a.fuse_kind) fob[rows[t] * NH + kz] = make_float2(f * z[t].x, f * z[t].y);
          }
        if (bin >= 0) {
          float w = (kz == 0 || 2 * kz == N) ? 1.0f : 2.0f;
          pk = p2 * (w01 * swin[kz] * w);
        }
      }
      // segmented inclusive scan over runs of equal bin (|k| grows with kz)
      int prev = __shfl_up_sync(0xffffffffu, bin, 1);
      bool head = lane == 0 || prev != bin;
      unsigned heads = __ballot_sync(0xffffffffu, head);
      unsigned below = heads & ((2u << lane) - 1u);
      int seg0 = 31 - __clz(below);
      float acc = pk;
      for (int o = 1; o < 32; o <<= 1) {
        float t = __shfl_up_sync(0xffffffffu, acc, o);
        if (lane - o >= seg0) acc += t;
      }
      int nbin = __shfl_down_sync(0xffffffffu, bin, 1);
      bool tail = lane == 31 || nbin != bin;
      if (tail && bin >= 0) {
        float old = a.priv ? shi[bin] : atomicAdd(&shi[bin], acc);
        float sum = old + acc, bp = sum - old, err = (old - (sum - bp)) + (acc - bp);
        if (a.priv) {
          shi[bin] = sum;
          slo[bin] += err;
        } else {
          atomicAdd(&slo[bin], err);
        }
      }
    }
  }
  __syncthreads();
  for (int b = threadIdx.x; b < nbins; b += blockDim.x) {
    double t = 0.0;
    for (int w = 0; w < nwb; w++) t += (double)shi0[w * nbins + b] + (double)slo0[w * nbins + b];
    bpb[(long long)blockIdx.x * nbins + b] = t;
  }
}

// Deterministic cross-block sum in FP64 (the MPI_Allreduce of compute_pofk.c:225).
__global__ void k_pofk_reduce(const double *__restrict__ block_part, int nblocks, int nbins, double *__restrict__ sums,
                              long long part_bs, long long sum_bs) {
  block_part += blockIdx.y * part_bs;
  sums += blockIdx.y * sum_bs;
  int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nbins) return;
  double s = 0.0;
  for (int k = 0; k < nblocks; k++) s += block_part[(long long)k * nbins + b];
  sums[b] = s;
}

static int launch_pofk(mgp_pofk_kargs ka, int nblocks, double *sums, cudaStream_t st, int nbox = 1,
                       long long sum_bs = 0) {
  ka.part_bs = (long long)nblocks * ka.nbins;
  const int h = ka.N / 2;
  ka.priv = (size_t)ka.nbins * (MGP_THREADS / 32) * 2 * sizeof(float) <= 96 * 1024;
  size_t shmem = 2 * sizeof(float) * (size_t)ka.nbins * (ka.priv ? MGP_THREADS / 32 : 1) +
                 (ka.thr ? sizeof(int) * (size_t)(ka.nbins + 1) : 0) + sizeof(float) * (size_t)(h + 1);
  if (shmem > 48 * 1024) {
    if (cudaFuncSetAttribute(k_pofk, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shmem) != cudaSuccess)
      return mgp_set_error(MGP_EINVAL, "P(k) needs %zu bytes of shared memory", shmem);
  }
  k_pofk<<<dim3(nblocks, nbox), MGP_THREADS, shmem, st>>>(ka);
  MGP_CHECK_LAUNCH();
  g_kernel_launches++;
  k_pofk_reduce<<<dim3((ka.nbins + 127) / 128, nbox), 128, 0, st>>>(ka.block_part, nblocks, ka.nbins, sums, ka.part_bs,
                                                                   sum_bs);
  MGP_CHECK_LAUNCH();
  g_kernel_launches++;
  return MGP_OK;
}

int mgp_launch_pofk(const float *dk, int N, const int *rk_bin, const float *win, int nbins, double *block_part,
                    int nblocks, double *sums, cudaStream_t st) {
  mgp_pofk_kargs ka;
  memset(&ka, 0, sizeof(ka));
  ka.dk = (const float2 *)dk;
  ka.N = N;
  ka.nbins = nbins;
  ka.rk_bin = rk_bin;
  ka.win = win;
  ka.block_part = block_part;
  return launch_pofk(ka, nblocks, sums, st);
}

int mgp_launch_pofk_thr(const float *dk, int N, const int *thr, const float *win, int nbins, int bintype, double kmin,
                        double kmax, double *block_part, int nblocks, double *sums, int fuse_kind, int filter,
                        float *fuse_out, float fuse_a, float fuse_b, cudaStream_t st, int nbox, long long g_bs,
                        long long sum_bs) {
  mgp_pofk_kargs ka;
  memset(&ka, 0, sizeof(ka));
  ka.dk = (const float2 *)dk;
  ka.N = N;
  ka.nbins = nbins;
  ka.bintype = bintype;
  ka.thr = thr;
  ka.win = win;
  ka.kmin = (float)kmin;
  ka.kmax = (float)kmax;
  ka.block_part = block_part;
  ka.fuse_kind = fuse_kind;
  ka.filter = filter;
  ka.fuse_out = (float2 *)fuse_out;
  ka.fuse_a = fuse_a;
  ka.fuse_b = fuse_b;
  ka.dk_bs = g_bs / 2;
  return launch_pofk(ka, nblocks, sums, st, nbox, sum_bs);
}

// ------------------------------------------------------------ force grids
// Forces (src/auxPM.c:437-535): F_a(k) = i k_a/k^2 * S(k) / N^3 with
// S = delta(k) [+ MG source], no CIC deconvolution, k = 0 zeroed.  Wave
// numbers: x index i > N/2 -> i - N (N/2 stays +N/2), y index j > N/2 is the
// reference's mirrored j (dd = -(N - j)), kz >= 0.
// MG source (auxPM.c:450-455): mg_kind 1 adds coupling * RK/(RK + m^2) *
// delta_eff(k) (EffDensitykToPhiofk, src/mg.h:74-116, fused here); mg_kind 2
// adds delta_eff(k) as is (density screening, src/mg.h:197-260); mg_kind 3
// scales delta by (1 + coupling) (DGP without screening, src/mg.h:209-215).
// On the kz = 0 and kz = N/2 planes a component whose own index sits on the
// Nyquist plane is odd under k -> -k with the same stored index, so it has no
// Hermitian partner; a real-output inverse FFT keeps only the Hermitian part
// there, which is zero.  Those entries are written as zero so that cuFFT and
// FFTW give the same real field.
__global__ void __launch_bounds__(MGP_THREADS) k_forces(const float2 *__restrict__ dk, const float2 *__restrict__ mgk,
                                                        float mg_coupling, float mg_mass2, int mg_kind, int N,
                                                        float cfac, float2 *__restrict__ fx, float2 *__restrict__ fy,
                                                        float2 *__restrict__ fz, long long g_bs,
                                                        const mgp_box_scalars *__restrict__ bs) {
  {
    // box blockIdx.y: input grids g_bs floats apart, the three force grids 3 g_bs
    const long long o = blockIdx.y * (g_bs / 2);
    dk += o;
    if (mgk) mgk += o;
    fx += 3 * o;
    fy += 3 * o;
    fz += 3 * o;
    if (bs) {
      mg_coupling = bs[blockIdx.y].coupling;
      mg_mass2 = bs[blockIdx.y].mass2;
    }
  }
  const int NH = N / 2 + 1;
  const long long total = (long long)N * N * NH;
  (void)total;
  const int lane = threadIdx.x & 31;
  const long long wid = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
  // one warp per (i, j) row of the half-complex grid, lanes along kz
  for (long long r = wid; r < (long long)N * N; r += nw) {
    const int i = (int)(r / N), j = (int)(r - (long long)i * N);
#pragma unroll 4
    for (int kz = lane; kz < NH; kz += 32) {
    const long long c = r * NH + kz;
    int dx = i > N / 2 ? i - N : i, dy = j > N / 2 ? j - N : j, dz = kz;
    int rk = dx * dx + dy * dy + dz * dz;
    float2 S = dk[c];
    if (mg_kind == 1) {
      float2 m = mgk[c];
      float f = mg_coupling * (float)rk / ((float)rk + mg_mass2);
      S.x = fmaf(f, m.x, S.x);
      S.y = fmaf(f, m.y, S.y);
    } else if (mg_kind == 2) {
      float2 m = mgk[c];
      S.x += m.x;
      S.y += m.y;
    } else if (mg_kind == 3) {
      S.x *= 1.0f + mg_coupling;
      S.y *= 1.0f + mg_coupling;
    }
    float g = rk == 0 ? 0.0f : cfac / (float)rk;  // = -1/(RK N^3 Scale)
    float ax = g * (float)dx, ay = g * (float)dy, az = g * (float)dz;
    if (kz == 0 || 2 * kz == N) {
      if (2 * i == N) ax = 0.0f;
      if (2 * j == N) ay = 0.0f;
      az = 0.0f;
    }
    fx[c] = make_float2(-ax * S.y, ax * S.x);
    fy[c] = make_float2(-ay * S.y, ay * S.x);
    fz[c] = make_float2(-az * S.y, az * S.x);
  }
  }
}

int mgp_launch_forces(const float *dk, const float *mgk, float mg_coupling, float mg_mass2, int mg_kind, int N,
                      double box, float *frc, long long grid_floats, cudaStream_t st, int nbox,
                      const mgp_box_scalars *bs) {
  const long long total = (long long)N * N * (N / 2 + 1);
  double scale = 2.0 * M_PI / box;
  float cfac = (float)(-1.0 / ((double)N * N * N * scale));
  float2 *fx = (float2 *)frc, *fy = (float2 *)(frc + grid_floats), *fz = (float2 *)(frc + 2 * grid_floats);
  k_forces<<<grid_boxes(total, g_budget_grid, nbox), MGP_THREADS, 0, st>>>((const float2 *)dk, (const float2 *)mgk, mg_coupling,
                                                               mg_mass2, mg_kind, N, cfac, fx, fy, fz, grid_floats, bs);
  MGP_CHECK_LAUNCH();
  g_kernel_launches++;
  return MGP_OK;
}

// ------------------------------------ fused MtoParticles + Kick + Drift
// MtoParticles (src/auxPM.c:560-644): trilinear interpolation of the three
// force grids at the particle; Kick (src/main.c:688-742):
//   v += dda * (-1.5 Omega (Disp - <Disp>) - UseCOLA (D1 ddD + D2 ddD2)/A);
// Drift (src/main.c:747-787):
//   x += (v - <v>) dyyy + UseCOLA (D1 dD + D2 dD2).
// The global means only shift all velocities (or all positions) by one
// vector, so the kernel applies the particle-local part and carries the
// uniform part in the FP64 offsets cv / cx (k_finalize_kd), which removes
// the two extra passes over the particles the reference makes.
__device__ __forceinline__ double block_sum_d(double v, double *sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) sh[w] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int k = 0; k < (int)(blockDim.x >> 5); k++) s += sh[k];
  return s;
}

// IDX is the grid offset type: 32-bit when the padded grid has < 2^31
// floats (N <= 1024), which keeps the 24-point gather in fewer registers.
// P2: Ns = 2^ls, lattice and cell index arithmetic by shifts (identical
// results).
template <typename IDX, bool P2>
__global__ void __launch_bounds__(MGP_THREADS, 4) k_interp_kick_drift(
    const float *__restrict__ frc, long long gf, int N, long long P, int Ns, long long np, float *__restrict__ s,
    float *__restrict__ v, const float *__restrict__ D1, const float *__restrict__ D2,
    const mgp_dstate *__restrict__ st, double *__restrict__ partials, mgp_kd_args a,
    const mgp_box_scalars *__restrict__ bs, int ls, const unsigned *__restrict__ qlat) {
  __shared__ double sh[MGP_THREADS / 32];
  {
    // box blockIdx.y of a batch: force grids 3 gf apart, particle arrays 3 np
    const int bx = blockIdx.y;
    frc += bx * 3 * gf;
    s += bx * 3 * np;
    v += bx * 3 * np;
    D1 += bx * 3 * a.lpt_stride;
    D2 += bx * 3 * a.lpt_stride;
    st += bx;
    partials += (long long)bx * gridDim.x * 6;
    if (bs) {
      a.kick_d1 = bs[bx].kick_d1;
      a.kick_d2 = bs[bx].kick_d2;
      a.dD1 = bs[bx].dD1;
      a.dD2 = bs[bx].dD2;
    }
  }
  const float ox = (float)(st->cx[0] * a.scale), oy = (float)(st->cx[1] * a.scale), oz = (float)(st->cx[2] * a.scale);
  const float *F0 = frc, *F1 = frc + gf, *F2 = frc + 2 * gf;
  const IDX Pi = (IDX)P, NPi = (IDX)N * (IDX)P;
  float accD[3] = {0.f, 0.f, 0.f}, accV[3] = {0.f, 0.f, 0.f};
  long long stride = (long long)gridDim.x * blockDim.x;
  const float inv_ns = 1.0f / (float)Ns;
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < np; p += stride) {
    // lattice point of the particle in slot p: qlat[p] when the arrays are
    // held in cell-tile order, else p itself
    const long long lat = qlat ? (long long)qlat[p] : p;
    int i, j, k;
    float sp[3] = {s[p], s[np + p], s[2 * np + p]};
    int ix, iy, iz;
    float DX, DY, DZ;
    if (P2) {
      lattice_ijk_p2((unsigned)lat, ls, i, j, k);
      cell_frac_p2(i, sp[0], ox, N, ls, inv_ns, a.scale, ix, DX);
      cell_frac_p2(j, sp[1], oy, N, ls, inv_ns, a.scale, iy, DY);
      cell_frac_p2(k, sp[2], oz, N, ls, inv_ns, a.scale, iz, DZ);
    } else {
      if (np <= 0xffffffffLL)
        lattice_ijk((unsigned)lat, Ns, i, j, k);
      else
        lattice_ijk(lat, Ns, i, j, k);
      cell_frac(i, sp[0], ox, N, Ns, a.scale, ix, DX);
      cell_frac(j, sp[1], oy, N, Ns, a.scale, iy, DY);
      cell_frac(k, sp[2], oz, N, Ns, a.scale, iz, DZ);
    }
    const float TX = 1.0f - DX, TY = 1.0f - DY, TZ = 1.0f - DZ;
    const IDX x0 = (IDX)ix * NPi, x1 = (ix + 1 == N ? 0 : (IDX)(ix + 1) * NPi);
    const IDX y0 = (IDX)iy * Pi, y1 = (iy + 1 == N ? 0 : (IDX)(iy + 1) * Pi);
    const IDX z0 = (IDX)iz, z1 = (iz + 1 == N ? 0 : (IDX)(iz + 1));
    const IDX o000 = x0 + y0 + z0, o001 = x0 + y0 + z1, o010 = x0 + y1 + z0, o011 = x0 + y1 + z1;
    const IDX o100 = x1 + y0 + z0, o101 = x1 + y0 + z1, o110 = x1 + y1 + z0, o111 = x1 + y1 + z1;
    const float w000 = TX * TY * TZ, w001 = TX * TY * DZ, w010 = TX * DY * TZ, w011 = TX * DY * DZ;
    const float w100 = DX * TY * TZ, w101 = DX * TY * DZ, w110 = DX * DY * TZ, w111 = DX * DY * DZ;
    float disp[3];
    const float *Fa[3] = {F0, F1, F2};
#pragma unroll
    for (int ax = 0; ax < 3; ax++) {
      const float *F = Fa[ax];
      disp[ax] = __ldg(F + o000) * w000 + __ldg(F + o001) * w001 + __ldg(F + o010) * w010 + __ldg(F + o011) * w011 +
                 __ldg(F + o100) * w100 + __ldg(F + o101) * w101 + __ldg(F + o110) * w110 + __ldg(F + o111) * w111;
    }
    // D1/D2 offsets: the lattice point for particle arrays (pitch Ns; they
    // stay in lattice order when s and v are in tile order), the lattice
    // point in the row-padded slot grids otherwise
    const long long od = a.lpt_pitch == Ns ? lat : ((long long)i * Ns + j) * a.lpt_pitch + k;
#pragma unroll
    for (int ax = 0; ax < 3; ax++) {
      long long o = ax * np + p;
      float d1 = D1[ax * a.lpt_stride + od], d2 = D2[ax * a.lpt_stride + od];
      float vn = v[o] + a.kick_disp * disp[ax] + a.kick_d1 * d1 + a.kick_d2 * d2;
      v[o] = vn;
      if (a.do_drift) s[o] = sp[ax] + vn * a.dyyy + a.dD1 * d1 + a.dD2 * d2;
      accD[ax] += disp[ax];
      accV[ax] += vn;
    }
  }
#pragma unroll
  for (int q = 0; q < 3; q++) {
    double t = block_sum_d((double)accD[q], sh);
    if (threadIdx.x == 0) partials[(long long)blockIdx.x * 6 + q] = t;
    t = block_sum_d((double)accV[q], sh);
    if (threadIdx.x == 0) partials[(long long)blockIdx.x * 6 + 3 + q] = t;
  }
}

// Means over all particles and offset update (one block, fixed order).
__global__ void k_finalize_kd(mgp_dstate *st, const double *__restrict__ partials, int nblocks, double inv_np,
                              double dda_omega, double dyyy, int do_drift) {
  __shared__ double sh[6][MGP_THREADS / 32];
  st += blockIdx.x;  // one block per box
  partials += (long long)blockIdx.x * nblocks * 6;
  double acc[6] = {0, 0, 0, 0, 0, 0};
  for (int b = threadIdx.x; b < nblocks; b += blockDim.x)
    for (int q = 0; q < 6; q++) acc[q] += partials[(long long)b * 6 + q];
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int q = 0; q < 6; q++) {
    double x = acc[q];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) sh[q][w] = x;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double t[6];
    for (int q = 0; q < 6; q++) {
      t[q] = 0.0;
      for (int k = 0; k < (int)(blockDim.x >> 5); k++) t[q] += sh[q][k];
    }
    for (int ax = 0; ax < 3; ax++) {
      double mD = t[ax] * inv_np, mV = t[3 + ax] * inv_np;
      st->mean_disp[ax] = mD;
      st->cv[ax] += dda_omega * mD;
      st->mean_v[ax] = mV;
      if (do_drift) st->cx[ax] -= mV * dyyy;
    }
  }
}

int mgp_ikd_blocks(long long np) { return blocks_for(np, 8); }

int mgp_launch_ikd(const float *frc, long long gf, int N, long long P, int Ns, long long np, float *s, float *v,
                   const float *D1, const float *D2, mgp_dstate *dst, double *partials, int nblocks,
                   const mgp_kd_args *a, cudaStream_t st, int nbox, const mgp_box_scalars *bs,
                   const unsigned *qlat) {
  const dim3 g(nblocks, nbox);
  const int ls = lattice_log2(Ns);
  const bool p2 = ls >= 0 && np <= 0xffffffffLL;
  if (gf < (1LL << 31) && p2)
    k_interp_kick_drift<int, true><<<g, MGP_THREADS, 0, st>>>(frc, gf, N, P, Ns, np, s, v, D1, D2, dst, partials, *a,
                                                              bs, ls, qlat);
  else if (gf < (1LL << 31))
    k_interp_kick_drift<int, false><<<g, MGP_THREADS, 0, st>>>(frc, gf, N, P, Ns, np, s, v, D1, D2, dst, partials, *a,
                                                               bs, ls, qlat);
  else if (p2)
    k_interp_kick_drift<long long, true><<<g, MGP_THREADS, 0, st>>>(frc, gf, N, P, Ns, np, s, v, D1, D2, dst, partials,
                                                                    *a, bs, ls, qlat);
  else
    k_interp_kick_drift<long long, false><<<g, MGP_THREADS, 0, st>>>(frc, gf, N, P, Ns, np, s, v, D1, D2, dst,
                                                                     partials, *a, bs, ls, qlat);
  MGP_CHECK_LAUNCH();
  g_kernel_launches++;
  k_finalize_kd<<<nbox, MGP_THREADS, 0, st>>>(dst, partials, nblocks, 1.0 / (double)np, a->dda_omega, a->dyyy_d,
                                              a->do_drift);
  MGP_CHECK_LAUNCH();
  g_kernel_launches++;
  return MGP_OK;
}

int mgp_launch_finalize_kd(mgp_dstate *dst, const double *partials, int nblocks, long long np, double dda_omega,
                           double dyyy, int do_drift, cudaStream_t st) {
  k_finalize_kd<<<1, MGP_THREADS, 0, st>>>(dst, partials, nblocks, 1.0 / (double)np, dda_omega, dyyy, do_drift);
  MGP_CHECK_LAUNCH();
  g_kernel_launches++;
  return MGP_OK;
}

// --------------------------------------------------------- MG passes
// DivideByLaplacian (src/mg.h:21-64): Phi_N(k) = -norm * delta(k) / RK.
__global__ void k_div_laplacian(const float2 *__restrict__ dk, float2 *__restrict__ out, int N, float norm,
                                long long g_bs) {
  dk += blockIdx.y * (g_bs / 2);
  out += blockIdx.y * (g_bs / 2);
  const int NH = N / 2 + 1;
  const long long total = (long long)N * N * NH;
  (void)total;
  const int lane = threadIdx.x & 31;
  const long long wid = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
  // one warp per (i, j) row of the half-complex grid, lanes along kz
  for (long long r = wid; r < (long long)N * N; r += nw) {
    const int i = (int)(r / N), j = (int)(r - (long long)i * N);
#pragma unroll 4
    for (int kz = lane; kz < NH; kz += 32) {
    const long long c = r * NH + kz;
    int d0 = i > N / 2 ? N - i : i, d1 = j > N / 2 ? N - j : j;
    int rk = d0 * d0 + d1 * d1 + kz * kz;
    float2 z = dk[c];
    const float f = mg_kfilter(rk, 2, 0, 0.0f, norm);
    out[c] = make_float2(f * z.x, f * z.y);
  }
  }
}

int mgp_launch_div_laplacian(const float *dk, float *out, int N, float norm, cudaStream_t st, int nbox,
                             long long g_bs) {
  const long long total = (long long)N * N * (N / 2 + 1);
  k_div_laplacian<<<grid_boxes(total, g_budget_grid, nbox), MGP_THREADS, 0, st>>>((const float2 *)dk, (float2 *)out, N, norm, g_bs);
  MGP_CHECK_LAUNCH();
  g_kernel_launches++;
  return MGP_OK;
}

// SmoothDensityField (src/mg.h:268-309) with smoothing_filter (mg.h:318-338).
__global__ void k_smooth(const float2 *__restrict__ dk, float2 *__restrict__ out, int N, int filter, float kR1,
                         float norm, long long g_bs) {
  dk += blockIdx.y * (g_bs / 2);
  out += blockIdx.y * (g_bs / 2);
  const int NH = N / 2 + 1;
  const long long total = (long long)N * N * NH;
  (void)total;
  const int lane = threadIdx.x & 31;
  const long long wid = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
  // one warp per (i, j) row of the half-complex grid, lanes along kz
  for (long long r = wid; r < (long long)N * N; r += nw) {
    const int i = (int)(r / N), j = (int)(r - (long long)i * N);
#pragma unroll 4
    for (int kz = lane; kz < NH; kz += 32) {
    const long long c = r * NH + kz;
    int d0 = i > N / 2 ? N - i : i, d1 = j > N / 2 ? N - j : j;
    int rk = d0 * d0 + d1 * d1 + kz * kz;
    const float f = mg_kfilter(rk, 1, filter, kR1, norm);
    float2 z = dk[c];
    out[c] = make_float2(f * z.x, f * z.y);
  }
  }
}

int mgp_launch_smooth(const float *dk, float *out, int N, int filter, float kR1, float norm, cudaStream_t st,
                      int nbox, long long g_bs) {
  const long long total = (long long)N * N * (N / 2 + 1);
  k_smooth<<<grid_boxes(total, g_budget_grid, nbox), MGP_THREADS, 0, st>>>((const float2 *)dk, (float2 *)out, N, filter, kR1, norm,
                                                               g_bs);
  MGP_CHECK_LAUNCH();
  g_kernel_launches++;
  return MGP_OK;
}

// Potential screening (src/mg.h:174-176, screening_factor_potential at
// src/user_defined_functions.h:725-750): rho *= min(1, |phicrit / Phi_N|)
// where Phi_N < 0, else 1.  Padding entries are included as in the reference.
__device__ __forceinline__ float screen_pot(float ph, float phicrit) {
  float f = 1.0f;
  if (ph < 0.0f) {
    f = fabsf(phicrit / ph);
    if (f > 1.0f) f = 1.0f;
  }
  return f;
}
__global__ void k_screen_potential(float *__restrict__ rho, const float *__restrict__ phi, long long n, float phicrit,
                                   const mgp_box_scalars *__restrict__ bs) {
  // box blockIdx.y: grids n floats apart
  rho += blockIdx.y * n;
  phi += blockIdx.y * n;
  if (bs) phicrit = bs[blockIdx.y].phicrit;
  long long stride = (long long)gridDim.x * blockDim.x;
  long long n4 = n >> 2;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += stride) {
    float4 r = reinterpret_cast<float4 *>(rho)[i], ph = reinterpret_cast<const float4 *>(phi)[i];
    r.x *= screen_pot(ph.x, phicrit);
    r.y *= screen_pot(ph.y, phicrit);
    r.z *= screen_pot(ph.z, phicrit);
    r.w *= screen_pot(ph.w, phicrit);
    reinterpret_cast<float4 *>(rho)[i] = r;
  }
  for (long long i = 4 * n4 + (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
    rho[i] *= screen_pot(phi[i], phicrit);
}

int mgp_launch_screen_potential(float *rho, const float *phi, long long n, float phicrit, cudaStream_t st, int nbox,
                                const mgp_box_scalars *bs) {
  k_screen_potential<<<grid_boxes(n, g_budget_grid, nbox), MGP_THREADS, 0, st>>>(rho, phi, n, phicrit, bs);
  MGP_CHECK_LAUNCH();
  g_kernel_launches++;
  return MGP_OK;
}

// Density screening (src/mg.h:241-250, screening_factor_density at
// src/user_defined_functions.h:757-773): rho *= coupling * 2(sqrt(1+f)-1)/f,
// f = pref (1 + delta_R), factor 1 when f < 1e-5.
__device__ __forceinline__ float screen_den(float dsm, float pref) {
  float fac = pref * (1.0f + dsm);
  return fac < 1e-5f ? 1.0f : 2.0f * (sqrtf(1.0f + fac) - 1.0f) / fac;
}
// base 1: rho *= 1 + coupling * S, i.e. the density plus its fifth-force
// source in one field (the force pass then reads one spectrum).
__global__ void k_screen_density(float *__restrict__ rho, const float *__restrict__ dsm, long long n, float coupling,
                                 float pref, const mgp_box_scalars *__restrict__ bs, float base) {
  // box blockIdx.y: grids n floats apart
  rho += blockIdx.y * n;
  dsm += blockIdx.y * n;
  if (bs) {
    coupling = bs[blockIdx.y].coupling;
    pref = bs[blockIdx.y].pref;
  }
  long long stride = (long long)gridDim.x * blockDim.x;
  long long n4 = n >> 2;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += stride) {
    float4 r = reinterpret_cast<float4 *>(rho)[i], d = reinterpret_cast<const float4 *>(dsm)[i];
    r.x *= fmaf(coupling, screen_den(d.x, pref), base);
    r.y *= fmaf(coupling, screen_den(d.y, pref), base);
    r.z *= fmaf(coupling, screen_den(d.z, pref), base);
    r.w *= fmaf(coupling, screen_den(d.w, pref), base);
    reinterpret_cast<float4 *>(rho)[i] = r;
  }
  for (long long i = 4 * n4 + (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
    rho[i] *= fmaf(coupling, screen_den(dsm[i], pref), base);
}

int mgp_launch_screen_density(float *rho, const float *dsm, long long n, float coupling, float pref, cudaStream_t st,
                              int nbox, const mgp_box_scalars *bs, float base) {
  k_screen_density<<<grid_boxes(n, g_budget_grid, nbox), MGP_THREADS, 0, st>>>(rho, dsm, n, coupling, pref, bs,
                                                                                base);
  MGP_CHECK_LAUNCH();
  g_kernel_launches++;
  return MGP_OK;
}

// A user's screening function (mgp_model_hooks), tabulated on the host once
// per step over t = asinh(u / u_s) at nt uniform points from t0: rho *=
// mult * S(u) with S interpolated linearly in t, u the Newtonian potential
// or the smoothed density at the cell (clamped to the table's range).
__global__ void k_screen_table(float *__restrict__ rho, const float *__restrict__ arg, long long n, float mult,
                               const float *__restrict__ tab, int nt, float inv_us, float t0, float inv_dt) {
  long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    float x = (asinhf(arg[i] * inv_us) - t0) * inv_dt;
    x = fminf(fmaxf(x, 0.0f), (float)(nt - 1));
    int j = min((int)x, nt - 2);
    float f = x - (float)j;
    float S = fmaf(f, tab[j + 1] - tab[j], tab[j]);
    rho[i] *= mult * S;
  }
}

int mgp_launch_screen_table(float *rho, const float *arg, long long n, float mult, const float *tab, int nt, double us,
                            double t0, double dt, cudaStream_t st) {
  k_screen_table<<<blocks_for(n, g_budget_grid), MGP_THREADS, 0, st>>>(rho, arg, n, mult, tab, nt, (float)(1.0 / us),
                                                                       (float)t0, (float)(1.0 / dt));
  MGP_CHECK_LAUNCH();
  g_kernel_launches++;
  return MGP_OK;
}

// ComputeFifthForce_TimeDepGeffModels (src/mg.h:127-137): P3D *= Geff/G.
__global__ void k_scale(float *__restrict__ c, long long n, float f) {
  long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) c[i] *= f;
}

int mgp_launch_scale_complex(float *c, long long ncomplex, float factor, cudaStream_t st) {
  k_scale<<<blocks_for(2 * ncomplex, 8), MGP_THREADS, 0, st>>>(c, 2 * ncomplex, factor);
  MGP_CHECK_LAUNCH();
  g_kernel_launches++;
  return MGP_OK;
}

// ------------------------------------------------------------------ IC
// displacement_fields, Gaussian branch (src/2LPT.c:276-495): one thread per
// (i, j) column of the k grid replays that column's white-noise stream
// (seeded by seedtable[i N + j], 2LPT.c:344) in the reference's draw order --
// phase, then amplitude unless amplitude-fixed -- and writes delta(k) for
// kz < N/2, including the Hermitian partners on the kz = 0 plane.
// amp_rk[RK] = Box^-1.5 sqrt(P(k) * rescale) is tabulated on the host in FP64;
// cut1d[|d|] is the cube cut of 2LPT.c:383-386 evaluated on the host with the
// reference's exact double expression.
__global__ void __launch_bounds__(MGP_THREADS) k_ic_delta(const uint32_t *__restrict__ seedtable,
                                                          const double *__restrict__ amp_rk,
                                                          const unsigned char *__restrict__ cut1d, int N, int Ns,
                                                          double box, int fixed, int inverted, int sphere,
                                                          float2 *__restrict__ dk) {
  long long col = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= (long long)N * N) return;
  const int NH = N / 2 + 1;
  int i = (int)(col / N), j = (int)(col % N);
  uint32_t seed = seedtable[col];
  uint64_t n = 0;
  const double twopi = 2 * 3.14159265358979323846;
  for (int k = 0; k < N / 2; k++) {
    double phase = mgp_uniform(seed, n++);
    double ampl = 1.0;
    if (!fixed) {
      do { ampl = mgp_uniform(seed, n++); } while (ampl == 0.0);
    }
    if (2 * i == N || 2 * j == N) continue;
    if (i == 0 && j == 0 && k == 0) continue;
    int di = i < N / 2 ? i : i - N, dj = j < N / 2 ? j : j - N, dkz = k;
    int ai = di < 0 ? -di : di, aj = dj < 0 ? -dj : dj;
    if (sphere) {
      double kx = (di < 0 ? -(N - i) * 2 * 3.14159265358979323846 / box : i * 2 * 3.14159265358979323846 / box);
      double ky = (dj < 0 ? -(N - j) * 2 * 3.14159265358979323846 / box : j * 2 * 3.14159265358979323846 / box);
      double kzv = k * 2 * 3.14159265358979323846 / box;
      double km = sqrt(kx * kx + ky * ky + kzv * kzv);
      if (km * box / twopi > Ns / 2) continue;
    } else {
      if (cut1d[ai] || cut1d[aj] || cut1d[dkz]) continue;
    }
    int rk = ai * ai + aj * aj + dkz * dkz;
    double delta = amp_rk[rk];
    if (!fixed) delta *= sqrt(-log(ampl));
    if (inverted) delta = -delta;
    float sn, cs;
    sincospif((float)(2.0 * phase), &sn, &cs);
    float re = (float)delta * cs, im = (float)delta * sn;
    if (k > 0) {
      dk[((long long)i * N + j) * NH + k] = make_float2(re, im);
    } else if (i == 0) {
      if (j >= N / 2) continue;
      dk[((long long)j) * NH] = make_float2(re, im);
      dk[((long long)(N - j)) * NH] = make_float2(re, -im);
    } else {
      if (i >= N / 2) continue;
      int ii = N - i, jj = (N - j) % N;
      dk[((long long)i * N + j) * NH] = make_float2(re, im);
      dk[((long long)ii * N + jj) * NH] = make_float2(re, -im);
    }
  }
  (void)twopi;
}

int mgp_launch_ic_delta(const uint32_t *seedtable, const double *amp_rk, const unsigned char *cut1d, int N, int Ns,
                        double box, int fixed, int inverted, int sphere, float *dk, cudaStream_t st) {
  long long cols = (long long)N * N;
  int nb = (int)((cols + MGP_THREADS - 1) / MGP_THREADS);
  k_ic_delta<<<nb, MGP_THREADS, 0, st>>>(seedtable, amp_rk, cut1d, N, Ns, box, fixed, inverted, sphere, (float2 *)dk);
  MGP_CHECK_LAUNCH();
  g_kernel_launches++;
  return MGP_OK;
}

// Massive neutrinos in the density (src/auxPM.c:383-428): delta(k) <-
// cdmfac delta(k) + nufac[|k|^2] delta_IC(k) with delta_IC the stored linear
// CDM+baryon field of the IC (cdelta_cdm); the k = 0 mode is left as it is.
// One warp per (i, j) row of the half-complex grid, lanes along kz; FP32
// arithmetic (the grids are FP32, and FP64 runs at a small fraction of the
// FP32 rate on this part).
__global__ void k_nu_add(float2 *__restrict__ dk, const float2 *__restrict__ dk0, int N, float cdmfac,
                         const float *__restrict__ nufac) {
  const int NH = N / 2 + 1;
  const int lane = threadIdx.x & 31;
  const long long wid = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
  for (long long r = wid; r < (long long)N * N; r += nw) {
    const int i = (int)(r / N), j = (int)(r - (long long)i * N);
    const int di = i > N / 2 ? N - i : i, dj = j > N / 2 ? N - j : j;
    const int r2 = di * di + dj * dj;
    for (int kz = lane; kz < NH; kz += 32) {
      if (r == 0 && kz == 0) continue;
      const long long c = r * NH + kz;
      const float f = nufac[r2 + kz * kz];
      const float2 a = dk[c], b = dk0[c];
      dk[c] = make_float2(fmaf(f, b.x, cdmfac * a.x), fmaf(f, b.y, cdmfac * a.y));
    }
  }
}

// The neutrino factor per integer |k|^2 (rk = 1 .. nrk-1; rk = 0 is 0):
// fac T_nu(k, a) / den[rk] at k = kfac sqrt(rk), T_nu the cubic Hermite in
// ln k of the transfer row (val, dval on the nodes x), clamped to the table
// as Lookup_GSL_2D_Spline does (src/wrappers.c:129-136).
__global__ void k_nu_table(float *__restrict__ tab, int nrk, double kfac, double fac, const double *__restrict__ x,
                           const double *__restrict__ val, const double *__restrict__ dval, int nx,
                           const double *__restrict__ den) {
  for (int rk = blockIdx.x * blockDim.x + threadIdx.x; rk < nrk; rk += gridDim.x * blockDim.x) {
    if (rk == 0) {
      tab[0] = 0.0f;
      continue;
    }
    double xv = log(kfac * sqrt((double)rk));
    xv = fmin(fmax(xv, x[0]), x[nx - 1]);
    int lo = 0, hi = nx - 1;
    while (hi - lo > 1) {
      const int m = (lo + hi) / 2;
      if (x[m] > xv) hi = m;
      else lo = m;
    }
    const double dx = x[lo + 1] - x[lo], t = (xv - x[lo]) / dx;
    const double T = (1 + 2 * t) * (1 - t) * (1 - t) * val[lo] + t * t * (3 - 2 * t) * val[lo + 1] +
                     t * (1 - t) * (1 - t) * dx * dval[lo] + t * t * (t - 1) * dx * dval[lo + 1];
    tab[rk] = (float)(fac * T / den[rk]);
  }
}

int mgp_launch_nu_table(float *tab, int nrk, double kfac, double fac, const double *x, const double *val,
                        const double *dval, int nx, const double *den, cudaStream_t st) {
  k_nu_table<<<blocks_for(nrk, 4), MGP_THREADS, 0, st>>>(tab, nrk, kfac, fac, x, val, dval, nx, den);
  MGP_CHECK_LAUNCH();
  g_kernel_launches++;
  return MGP_OK;
}

int mgp_launch_nu_add(float *dk, const float *dk0, int N, double cdmfac, const float *nufac, cudaStream_t st) {
  const long long rows = (long long)N * N;
  k_nu_add<<<blocks_for(rows * 32, 8), MGP_THREADS, 0, st>>>((float2 *)dk, (const float2 *)dk0, N, (float)cdmfac,
                                                             nufac);
  MGP_CHECK_LAUNCH();
  g_kernel_launches++;
  return MGP_OK;
}

// ProcessParticlesSingleFile (src/readICfromfile.c:133-219): CIC of particles
// at positions in [0,1) of the box (FP64, [n][3]) onto a density grid pre-set
// to -1, with WPAR = (N/Ns)^3 folded into the y factors; a cell index that
// reaches N (position rounded up to the box edge) wraps to 0, as the
// reference's ghost slice does for x.
__global__ void k_cic_unit(const double *__restrict__ pos, long long n, int N, long long P, float wpar,
                           float *__restrict__ rho) {
  long long stride = (long long)gridDim.x * blockDim.x;
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += stride) {
    const double X = pos[3 * q] * N, Y = pos[3 * q + 1] * N, Z = pos[3 * q + 2] * N;
    unsigned IX = (unsigned)X, IY = (unsigned)Y, IZ = (unsigned)Z;
    const float DX = (float)(X - (double)IX), DZ = (float)(Z - (double)IZ);
    const float DYr = (float)(Y - (double)IY);
    const float TX = 1.f - DX, TZ = 1.f - DZ, TY = (1.f - DYr) * wpar, DY = DYr * wpar;
    if (IX >= (unsigned)N) IX = 0;
    if (IY >= (unsigned)N) IY = 0;
    if (IZ >= (unsigned)N) IZ = 0;
    const unsigned IXn = IX + 1 >= (unsigned)N ? 0 : IX + 1, IYn = IY + 1 >= (unsigned)N ? 0 : IY + 1,
                   IZn = IZ + 1 >= (unsigned)N ? 0 : IZ + 1;
    const long long x0 = (long long)IX * N, x1 = (long long)IXn * N;
    atomicAdd(rho + (x0 + IY) * P + IZ, TX * TY * TZ);
    atomicAdd(rho + (x0 + IY) * P + IZn, TX * TY * DZ);
    atomicAdd(rho + (x0 + IYn) * P + IZ, TX * DY * TZ);
    atomicAdd(rho + (x0 + IYn) * P + IZn, TX * DY * DZ);
    atomicAdd(rho + (x1 + IY) * P + IZ, DX * TY * TZ);
    atomicAdd(rho + (x1 + IY) * P + IZn, DX * TY * DZ);
    atomicAdd(rho + (x1 + IYn) * P + IZ, DX * DY * TZ);
    atomicAdd(rho + (x1 + IYn) * P + IZn, DX * DY * DZ);
  }
}

int mgp_launch_cic_unit(const double *pos, long long n, int N, long long P, float wpar, float *rho, cudaStream_t st) {
  k_cic_unit<<<blocks_for(n, 8), MGP_THREADS, 0, st>>>(pos, n, N, P, wpar, rho);
  MGP_CHECK_LAUNCH();
  g_kernel_launches++;
  return MGP_OK;
}

// delta(k) of a particle density as the linear field at z = 0
// (src/readICfromfile.c:640-676, 701-777): times normfac = D_LCDM(1) /
// D_LCDM(a_i) / N^3; modes with |d| > Ns/2 zeroed when N > Ns (for N <= Ns the
// three Nyquist planes, whose sign conventions differ between the
// reference's displacement and gradient passes); the CIC window divided out
// (gc[|d|] = 1/sinc^2(pi d/N) per axis) and the P(k) rescaling per integer
// |k|^2; the k = 0 mode zeroed.  In place on [N][N][N/2+1].
__global__ void k_ic_from_density(float2 *__restrict__ dk, int N, int Ns, double normfac,
                                  const double *__restrict__ gc, const double *__restrict__ rescale) {
  const int NH = N / 2 + 1;
  const long long n = (long long)N * N * NH;
  const long long cut2 = (long long)(Ns / 2) * (Ns / 2);
  long long stride = (long long)gridDim.x * blockDim.x;
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += stride) {
    const int kz = (int)(q % NH);
    const long long r = q / NH;
    const int j = (int)(r % N), i = (int)(r / N);
    const int di = i > N / 2 ? N - i : i, dj = j > N / 2 ? N - j : j;  // |d| per axis
    const long long d2 = (long long)di * di + (long long)dj * dj + (long long)kz * kz;
    const bool zero = d2 == 0 || (N > Ns && d2 > cut2) ||
                      (N <= Ns && (2 * i == N || 2 * j == N || 2 * kz == N));
    const double f = zero ? 0.0 : normfac * gc[di] * gc[dj] * gc[kz] * rescale[d2];
    float2 v = dk[q];
    v.x = (float)(f * v.x);
    v.y = (float)(f * v.y);
    dk[q] = v;
  }
}

int mgp_launch_ic_from_density(float *dk, int N, int Ns, double normfac, const double *gc, const double *rescale,
                               cudaStream_t st) {
  const long long n = (long long)N * N * (N / 2 + 1);
  k_ic_from_density<<<blocks_for(n, 8), MGP_THREADS, 0, st>>>((float2 *)dk, N, Ns, normfac, gc, rescale);
  MGP_CHECK_LAUNCH();
  g_kernel_launches++;
  return MGP_OK;
}

// Integer wave number of index idx in the IC convention (2LPT.c:359-375):
// idx < N/2 -> idx, else idx - N (so N/2 maps to -N/2).
__device__ __forceinline__ int ic_d(int idx, int N) { return idx < N / 2 ? idx : idx - N; }

// Displacement gradients (src/2LPT.c:1224-1270): psi_ab(k) = i k_b * Psi_a(k)
// = -k_a k_b / k^2 delta(k); order (00, 01, 02, 11, 12, 22).
__global__ void k_ic_grad6(const float2 *__restrict__ dk, float *__restrict__ out, long long gf, int N) {
  const int NH = N / 2 + 1;
  const long long total = (long long)N * N * NH;
  (void)total;
  const int lane = threadIdx.x & 31;
  const long long wid = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
  // one warp per (i, j) row of the half-complex grid, lanes along kz
  for (long long r = wid; r < (long long)N * N; r += nw) {
    const int i = (int)(r / N), j = (int)(r - (long long)i * N);
#pragma unroll 4
    for (int kz = lane; kz < NH; kz += 32) {
    const long long c = r * NH + kz;
    int d[3] = {ic_d(i, N), ic_d(j, N), ic_d(kz, N)};
    int rk = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
    float2 z = dk[c];
    float inv = rk == 0 ? 0.0f : -1.0f / (float)rk;
    const int A[6] = {0, 0, 0, 1, 1, 2}, B[6] = {0, 1, 2, 1, 2, 2};
#pragma unroll
    for (int g = 0; g < 6; g++) {
      float f = inv * (float)(d[A[g]] * d[B[g]]);
      ((float2 *)(out + g * gf))[c] = make_float2(f * z.x, f * z.y);
    }
  }
  }
}

int mgp_launch_ic_grad6(const float *dk, float *out6, long long gf, int N, cudaStream_t st) {
  const long long total = (long long)N * N * (N / 2 + 1);
  k_ic_grad6<<<blocks_for(total, 8), MGP_THREADS, 0, st>>>((const float2 *)dk, out6, gf, N);
  MGP_CHECK_LAUNCH();
  g_kernel_launches++;
  return MGP_OK;
}

// Second-order source in real space (src/2LPT.c:1282-1290), written over
// the psi_11 grid.
__global__ void k_ic_source(float *__restrict__ g, long long gf, long long n) {
  long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    float p00 = g[i], p01 = g[gf + i], p02 = g[2 * gf + i], p11 = g[3 * gf + i], p12 = g[4 * gf + i],
          p22 = g[5 * gf + i];
    g[3 * gf + i] = p00 * (p11 + p22) + p11 * p22 - p01 * p01 - p02 * p02 - p12 * p12;
  }
}

int mgp_launch_ic_source(float *g6, long long gf, int N, long long P, cudaStream_t st) {
  long long n = (long long)N * N * P;
  k_ic_source<<<blocks_for(n, 8), MGP_THREADS, 0, st>>>(g6, gf, n);
  MGP_CHECK_LAUNCH();
  g_kernel_launches++;
  return MGP_OK;
}

// ZA and 2LPT displacement fields in k space (src/2LPT.c:406-425,
// 1343-1355): Psi1_a = i k_a/k^2 delta, Psi2_a = -i k_a/k^2 S2, k in
// physical units (Box/2pi factor), IC sign convention.  Derivative-type
// Nyquist entries of the kz = 0 / N/2 planes are zeroed (see k_forces).
__global__ void k_ic_disp(const float2 *__restrict__ dk, const float *__restrict__ src_grid, float *__restrict__ out,
                          long long gf, int N, float box_over_2pi) {
  const int NH = N / 2 + 1;
  const long long total = (long long)N * N * NH;
  (void)total;
  const int lane = threadIdx.x & 31;
  const long long wid = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
  // one warp per (i, j) row of the half-complex grid, lanes along kz
  for (long long r = wid; r < (long long)N * N; r += nw) {
    const int i = (int)(r / N), j = (int)(r - (long long)i * N);
#pragma unroll 4
    for (int kz = lane; kz < NH; kz += 32) {
    const long long c = r * NH + kz;
    int d[3] = {ic_d(i, N), ic_d(j, N), ic_d(kz, N)};
    int rk = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
    float2 z = dk[c];
    float2 S = ((const float2 *)src_grid)[c];
    float inv = rk == 0 ? 0.0f : box_over_2pi / (float)rk;
    bool edge = (kz == 0 || 2 * kz == N);
#pragma unroll
    for (int a = 0; a < 3; a++) {
      float f = inv * (float)d[a];
      if (edge && ((a == 0 && 2 * i == N) || (a == 1 && 2 * j == N) || a == 2)) f = 0.0f;
      ((float2 *)(out + a * gf))[c] = make_float2(-f * z.y, f * z.x);
      ((float2 *)(out + (3 + a) * gf))[c] = make_float2(f * S.y, -f * S.x);
    }
  }
  }
}

int mgp_launch_ic_disp(const float *dk, const float *src, float *out6, long long gf, int N, double box,
                       cudaStream_t st) {
  // out6 must not alias dk; the source grid may be one of the six outputs:
  // each thread reads it before writing the same element.
  const long long total = (long long)N * N * (N / 2 + 1);
  k_ic_disp<<<blocks_for(total, 8), MGP_THREADS, 0, st>>>((const float2 *)dk, src, out6, gf, N,
                                                          (float)(box / (2.0 * M_PI)));
  MGP_CHECK_LAUNCH();
  g_kernel_launches++;
  return MGP_OK;
}

// Read-out of the six real displacement grids at the Lagrangian lattice
// (src/2LPT.c:1424-1491): trilinear with exact lattice fractions.
__global__ void __launch_bounds__(MGP_THREADS) k_ic_readout(const float *__restrict__ g, long long gf, int N, long long P,
                                                            int Ns, float *__restrict__ D1, float *__restrict__ D2,
                                                            float d2fac, double *__restrict__ partials) {
  __shared__ double sh[MGP_THREADS / 32];
  const long long np = (long long)Ns * Ns * Ns;
  float acc[6] = {0, 0, 0, 0, 0, 0};
  long long stride = (long long)gridDim.x * blockDim.x;
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < np; p += stride) {
    int li[3];
    lattice_ijk(p, Ns, li[0], li[1], li[2]);
    int c0[3], c1[3];
    float f[3];
    for (int a = 0; a < 3; a++) {
      long long qn = (long long)li[a] * N;
      int q = (int)(qn / Ns);
      f[a] = (float)(qn - (long long)q * Ns) / (float)Ns;
      if (q == N) q = N - 1;
      c0[a] = q;
      c1[a] = q + 1 >= N ? q + 1 - N : q + 1;
    }
    float w[8];
    long long id[8];
    for (int t = 0; t < 8; t++) {
      int bx = (t >> 2) & 1, by = (t >> 1) & 1, bz = t & 1;
      w[t] = (bx ? f[0] : 1.0f - f[0]) * (by ? f[1] : 1.0f - f[1]) * (bz ? f[2] : 1.0f - f[2]);
      id[t] = ((long long)(bx ? c1[0] : c0[0]) * N + (by ? c1[1] : c0[1])) * P + (bz ? c1[2] : c0[2]);
    }
    for (int a = 0; a < 3; a++) {
      float d1 = 0.f, d2 = 0.f;
      for (int t = 0; t < 8; t++) {
        d1 += g[a * gf + id[t]] * w[t];
        d2 += g[(3 + a) * gf + id[t]] * w[t];
      }
      d2 *= d2fac;
      D1[a * np + p] = d1;
      D2[a * np + p] = d2;
      acc[a] += d1;
      acc[3 + a] += d2;
    }
  }
  for (int q = 0; q < 6; q++) {
    double t = block_sum_d((double)acc[q], sh);
    if (threadIdx.x == 0) partials[(long long)blockIdx.x * 6 + q] = t;
  }
}

int mgp_launch_ic_readout(const float *g6, long long gf, int N, long long P, int Ns, float *D1, float *D2,
                          double *partials, int nblocks, cudaStream_t st) {
  float d2fac = (float)(-3.0 / 7.0 / ((double)N * N * N));
  k_ic_readout<<<nblocks, MGP_THREADS, 0, st>>>(g6, gf, N, P, Ns, D1, D2, d2fac, partials);
  MGP_CHECK_LAUNCH();
  g_kernel_launches++;
  return MGP_OK;
}

// Mean removal (2LPT.c:1493-1508) and initial state (main.c:257-309):
// s = D1 Di + D2 Di2 (displacement from q); v = D1 vD + D2 vD2, with
// vD = vD2 = 0 for COLA and dD/dy, dD2/dy at a_i without it (the 2LPT
// velocity, main.c:276-283).
__global__ void k_ic_finish(float *__restrict__ D1, float *__restrict__ D2, float *__restrict__ s, float *__restrict__ v,
                            long long np, const double *__restrict__ partials, int nblocks, float Di, float Di2,
                            float vD, float vD2) {
  __shared__ float mean[6];
  if (threadIdx.x < 6) {
    double t = 0.0;
    for (int b = 0; b < nblocks; b++) t += partials[(long long)b * 6 + threadIdx.x];
    mean[threadIdx.x] = (float)(t / (double)np);
  }
  __syncthreads();
  long long stride = (long long)gridDim.x * blockDim.x;
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < np; p += stride) {
    for (int a = 0; a < 3; a++) {
      long long o = a * np + p;
      float d1 = D1[o] - mean[a], d2 = D2[o] - mean[3 + a];
      D1[o] = d1;
      D2[o] = d2;
      s[o] = d1 * Di + d2 * Di2;
      v[o] = d1 * vD + d2 * vD2;
    }
  }
}

int mgp_launch_ic_finish(float *D1, float *D2, float *s, float *v, long long np, const double *partials, int nblocks,
                         float Di, float Di2, float vD, float vD2, cudaStream_t st) {
  k_ic_finish<<<blocks_for(np, 8), MGP_THREADS, 0, st>>>(D1, D2, s, v, np, partials, nblocks, Di, Di2, vD, vD2);
  MGP_CHECK_LAUNCH();
  g_kernel_launches++;
  return MGP_OK;
}

// ---------------------------------------------------- particle export
// Absolute positions wrap(q + s + cx) and velocities v + cv, AoS [np][3].
// FP32 arithmetic: the outputs are FP32 and the wrap needs no division.
__device__ __forceinline__ float wrap_box(float x, float box) {
  x -= box * floorf(x / box);  // no loop: bounded work for any input
  if (x >= box) x -= box;
  if (x < 0.0f) x += box;
  return (x >= box || x < 0.0f) ? 0.0f : x;
}

__global__ void k_positions(const float *__restrict__ s, const float *__restrict__ v, const mgp_dstate *__restrict__ st,
                            long long np, int Ns, double box, float *__restrict__ pos, float *__restrict__ vel) {
  long long stride = (long long)gridDim.x * blockDim.x;
  const float dq = (float)(box / (double)Ns), fbox = (float)box;
  const float cx[3] = {(float)st->cx[0], (float)st->cx[1], (float)st->cx[2]};
  const float cv[3] = {(float)st->cv[0], (float)st->cv[1], (float)st->cv[2]};
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < np; p += stride) {
    int li[3];
    if (np <= 0xffffffffLL)
      lattice_ijk((unsigned)p, Ns, li[0], li[1], li[2]);
    else
      lattice_ijk(p, Ns, li[0], li[1], li[2]);
    for (int a = 0; a < 3; a++) {
      if (pos) pos[3 * p + a] = wrap_box((float)li[a] * dq + (s[a * np + p] + cx[a]), fbox);
      if (vel) vel[3 * p + a] = v[a * np + p] + cv[a];
    }
  }
}

int mgp_launch_positions(const float *s, const mgp_dstate *dst, long long np, int Ns, double box, float *out_pos,
                         float *out_vel, const float *v, cudaStream_t st) {
  k_positions<<<blocks_for(np, 8), MGP_THREADS, 0, st>>>(s, v, dst, np, Ns, box, out_pos, out_vel);
  MGP_CHECK_LAUNCH();
  g_kernel_launches++;
  return MGP_OK;
}

// Import absolute AoS positions/velocities: s = nearest-image (pos - q).
__global__ void k_set_state(float *__restrict__ s, float *__restrict__ v, const float *__restrict__ pos,
                            const float *__restrict__ vel, long long np, int Ns, double box, long long p0,
                            long long p1) {
  long long stride = (long long)gridDim.x * blockDim.x;
  const float dq = (float)(box / (double)Ns), fbox = (float)box, half = 0.5f * (float)box;
  for (long long p = p0 + (long long)blockIdx.x * blockDim.x + threadIdx.x; p < p1; p += stride) {
    int li[3];
    if (np <= 0xffffffffLL)
      lattice_ijk((unsigned)p, Ns, li[0], li[1], li[2]);
    else
      lattice_ijk(p, Ns, li[0], li[1], li[2]);
    for (int a = 0; a < 3; a++) {
      if (pos) {
        float d = pos[3 * p + a] - (float)li[a] * dq;
        if (d > half) d -= fbox;
        if (d < -half) d += fbox;
        s[a * np + p] = d;
      }
      if (vel) v[a * np + p] = vel[3 * p + a];
    }
  }
}

int mgp_launch_set_state(float *s, float *v, const float *pos, const float *vel, long long np, int Ns, double box,
                         cudaStream_t st) {
  return mgp_launch_set_state_range(s, v, pos, vel, np, Ns, box, 0, np, st);
}

// particles p0 .. p1-1 only (the host-buffer step converts each uploaded chunk)
int mgp_launch_set_state_range(float *s, float *v, const float *pos, const float *vel, long long np, int Ns,
                               double box, long long p0, long long p1, cudaStream_t st) {
  if (p1 <= p0) return MGP_OK;
  k_set_state<<<blocks_for(p1 - p0, 8), MGP_THREADS, 0, st>>>(s, v, pos, vel, np, Ns, box, p0, p1);
  MGP_CHECK_LAUNCH();
  g_kernel_launches++;
  return MGP_OK;
}

// AoS [np][3] <-> SoA [3][np] for the host particle interface.
__global__ void k_aos_to_soa(const float *__restrict__ in, float *__restrict__ out, long long np) {
  long long stride = (long long)gridDim.x * blockDim.x;
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < np; p += stride)
    for (int a = 0; a < 3; a++) out[a * np + p] = in[3 * p + a];
}
int mgp_launch_aos_to_soa(const float *in, float *out, long long np, cudaStream_t st) {
  k_aos_to_soa<<<blocks_for(np, 4), MGP_THREADS, 0, st>>>(in, out, np);
  MGP_CHECK_LAUNCH();
  g_kernel_launches++;
  return MGP_OK;
}

// Particle data as written by Output (src/main.c:913-977): positions times
// lengthfac, velocities velfac * Hubble/A^1.5 * (Vel - <Vel> + UseCOLA (D1
// dD/dy + D2 dD2/dy)).  Vel - <Vel> equals the stored v minus its mean.
__global__ void k_output(const float *__restrict__ s, const float *__restrict__ v, const float *__restrict__ D1,
                         const float *__restrict__ D2, long long lstride, int lpitch,
                         const mgp_dstate *__restrict__ st, long long np, int Ns, double box, double lengthfac,
                         double vfac, double dDdy, double dD2dy, double cola, float *__restrict__ pos,
                         float *__restrict__ vel) {
  long long stride = (long long)gridDim.x * blockDim.x;
  const float dq = (float)(box / (double)Ns), fbox = (float)box, lf = (float)lengthfac, vf = (float)vfac;
  const float g1 = (float)(cola * dDdy), g2 = (float)(cola * dD2dy);
  const float cx[3] = {(float)st->cx[0], (float)st->cx[1], (float)st->cx[2]};
  const float mv[3] = {(float)st->mean_v[0], (float)st->mean_v[1], (float)st->mean_v[2]};
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < np; p += stride) {
    int li[3];
    lattice_ijk(p, Ns, li[0], li[1], li[2]);
    const long long od = ((long long)li[0] * Ns + li[1]) * lpitch + li[2];
    for (int a = 0; a < 3; a++) {
      long long o = a * np + p;
      pos[3 * p + a] = lf * wrap_box((float)li[a] * dq + (s[o] + cx[a]), fbox);
      vel[3 * p + a] = vf * ((v[o] - mv[a]) + D1[a * lstride + od] * g1 + D2[a * lstride + od] * g2);
    }
  }
}

int mgp_launch_output(const float *s, const float *v, const float *D1, const float *D2, long long lpt_stride,
                      int lpt_pitch, const mgp_dstate *dst, long long np, int Ns, double box, double lengthfac,
                      double vfac, double dDdy, double dD2dy, double cola, float *pos, float *vel, cudaStream_t st) {
  k_output<<<blocks_for(np, 4), MGP_THREADS, 0, st>>>(s, v, D1, D2, lpt_stride, lpt_pitch, dst, np, Ns, box,
                                                      lengthfac, vfac, dDdy, dD2dy, cola, pos, vel);
  MGP_CHECK_LAUNCH();
  g_kernel_launches++;
  return MGP_OK;
}

// ------------------------------------------------------ RSD multipoles
// PtoMesh_RSD (src/compute_pofk.c:280-393): CIC in redshift space with the
// line of sight mapped onto the grid's third axis (y LOS: grid axes (x, z, y);
// z LOS: (x, y, z)); the LOS coordinate moves by V * vnorm cells with
// V = Vel + UseCOLA (D1 dD/dy + D2 dD2/dy) (the reference does not subtract
// the mean velocity here) and wraps periodically.
__global__ void __launch_bounds__(MGP_THREADS) k_cic_rsd(const float *__restrict__ s, const float *__restrict__ v,
                                                         const float *__restrict__ D1, const float *__restrict__ D2,
                                                         long long lstride, int lpitch,
                                                         const mgp_dstate *__restrict__ st, long long np, int Ns,
                                                         int N, float scale, float wpar, int axis, float vnorm,
                                                         float g1, float g2, float *__restrict__ rho, long long P) {
  const int map[2][3] = {{0, 2, 1}, {0, 1, 2}};  // grid axis g takes particle axis map[.][g]
  const int *m = map[axis == 1 ? 0 : 1];
  float off[3];
  for (int g = 0; g < 3; g++) off[g] = (float)(st->cx[m[g]] * scale);
  const float cvl = (float)st->cv[m[2]];
  long long stride = (long long)gridDim.x * blockDim.x;
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < np; p += stride) {
    int li[3];
    lattice_ijk(p, Ns, li[0], li[1], li[2]);
    const long long ol = m[2] * np + p;
    const long long od = m[2] * lstride + ((long long)li[0] * Ns + li[1]) * lpitch + li[2];
    float V = (v[ol] + cvl) + D1[od] * g1 + D2[od] * g2;
    int ix, iy, iz;
    float DX, DY, DZ;
    cell_frac(li[m[0]], s[m[0] * np + p], off[0], N, Ns, scale, ix, DX);
    cell_frac(li[m[1]], s[m[1] * np + p], off[1], N, Ns, scale, iy, DY);
    cell_frac(li[m[2]], s[ol], off[2] + V * vnorm, N, Ns, scale, iz, DZ);
    float TX = 1.0f - DX, TY = (1.0f - DY) * wpar, TZ = 1.0f - DZ;
    DY *= wpar;
    int ixn = ix + 1 == N ? 0 : ix + 1, iyn = iy + 1 == N ? 0 : iy + 1, izn = iz + 1 == N ? 0 : iz + 1;
    long long r00 = ((long long)ix * N + iy) * P, r01 = ((long long)ix * N + iyn) * P;
    long long r10 = ((long long)ixn * N + iy) * P, r11 = ((long long)ixn * N + iyn) * P;
    atomicAdd(rho + r00 + iz, TX * TY * TZ);
    atomicAdd(rho + r00 + izn, TX * TY * DZ);
    atomicAdd(rho + r01 + iz, TX * DY * TZ);
    atomicAdd(rho + r01 + izn, TX * DY * DZ);
    atomicAdd(rho + r10 + iz, DX * TY * TZ);
    atomicAdd(rho + r10 + izn, DX * TY * DZ);
    atomicAdd(rho + r11 + iz, DX * DY * TZ);
    atomicAdd(rho + r11 + izn, DX * DY * DZ);
  }
}

int mgp_launch_cic_rsd(const float *s, const float *v, const float *D1, const float *D2, long long lpt_stride,
                       int lpt_pitch, const mgp_dstate *st, long long np, int Ns, int N, double box, float wpar,
                       int axis, float vnorm, float g1, float g2, float *rho, long long P, cudaStream_t stream) {
  k_cic_rsd<<<blocks_for(np, 8), MGP_THREADS, 0, stream>>>(s, v, D1, D2, lpt_stride, lpt_pitch, st, np, Ns, N,
                                                           (float)(N / box), wpar, axis, vnorm, g1, g2, rho, P);
  MGP_CHECK_LAUNCH();
  g_kernel_launches++;
  return MGP_OK;
}

// bin_up_RSD_power_spectrum (src/compute_pofk.c:518-753): sums of P, P mu^2
// and P mu^4 per bin with mu = kz/|k| (kz is the LOS index), mu = 0 for the
// k = 0 mode; FP64 shared-memory bins (used at output time only).
__global__ void __launch_bounds__(MGP_THREADS) k_pofk_mu(const float2 *__restrict__ dk, int N,
                                                         const int *__restrict__ rk_bin, const float *__restrict__ win,
                                                         int nbins, double *__restrict__ block_part) {
  extern __shared__ double smu[];
  const int NH = N / 2 + 1, h = N / 2;
  for (int b = threadIdx.x; b < 3 * nbins; b += blockDim.x) smu[b] = 0.0;
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const long long wid = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
  for (long long r = wid; r < (long long)N * N; r += nw) {
    const int i = (int)(r / N), j = (int)(r - (long long)i * N);
    const int d0 = i > h ? N - i : i, d1 = j > h ? N - j : j;
    for (int kz = lane; kz < NH; kz += 32) {
      const int rk = d0 * d0 + d1 * d1 + kz * kz;
      const int bin = rk_bin[rk];
      if (bin < 0) continue;
      float2 z = dk[r * NH + kz];
      double w = (kz == 0 || 2 * kz == N) ? 1.0 : 2.0;
      double pk = (double)(z.x * z.x + z.y * z.y) * (double)(win[d0] * win[d1] * win[kz]) * w;
      double mu2 = rk == 0 ? 0.0 : (double)(kz * kz) / (double)rk;
      atomicAdd(&smu[bin], pk);
      atomicAdd(&smu[nbins + bin], pk * mu2);
      atomicAdd(&smu[2 * nbins + bin], pk * mu2 * mu2);
    }
  }
  __syncthreads();
  for (int b = threadIdx.x; b < 3 * nbins; b += blockDim.x) block_part[(long long)blockIdx.x * 3 * nbins + b] = smu[b];
}

int mgp_launch_pofk_mu(const float *dk, int N, const int *rk_bin, const float *win, int nbins, double *block_part,
                       int nblocks, double *sums, cudaStream_t st) {
  size_t shmem = sizeof(double) * 3 * (size_t)nbins;
  if (shmem > 48 * 1024) {
    if (cudaFuncSetAttribute(k_pofk_mu, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shmem) != cudaSuccess)
      return mgp_set_error(MGP_EINVAL, "RSD P(k) needs %zu bytes of shared memory", shmem);
  }
  k_pofk_mu<<<nblocks, MGP_THREADS, shmem, st>>>((const float2 *)dk, N, rk_bin, win, nbins, block_part);
  MGP_CHECK_LAUNCH();
  g_kernel_launches++;
  k_pofk_reduce<<<(3 * nbins + 127) / 128, 128, 0, st>>>(block_part, nblocks, 3 * nbins, sums, 0, 0);
  MGP_CHECK_LAUNCH();
  g_kernel_launches++;
  return MGP_OK;
}
