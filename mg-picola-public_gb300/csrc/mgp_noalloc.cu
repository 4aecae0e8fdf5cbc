// P(k) shell binning without any allocation.
//
// Some callers cannot allocate device memory: code that runs inside another
// framework's memory pool or allocator hooks, callers that must not
// synchronise the device (cudaMalloc/cudaFree can), or code paths that run
// while a host-side memory budget is frozen.  mgp_pofk_noalloc serves them:
// it bins a caller-owned delta(k) grid exactly like mgp_pofk, but every
// scratch buffer it needs (bin table, window table, per-block partial sums,
// mode counts, results) lives in one file-scope device array of fixed size,
// so it calls no cudaMalloc, cudaFree or allocating library routine.
//
// Limits: Nmesh <= MGP_NA_MAX_N and at most MGP_NA_MAX_BINS bins after the
// reference's parameter adjustment; larger requests fail with MGP_EINVAL.
// The array (MGP_NA_SCRATCH_BYTES) is held on every device that loads the
// library until the process exits.  Every call shares it and it keeps the
// previous call's contents, so each call clears what must start at zero;
// calls whose GPU work overlaps (other host threads, other streams) race on
// it and must be serialised by the caller.  The array's device address is
// looked up by the first call on each device and kept for the process: after
// a cudaDeviceReset of that device the kept address is stale, so the entry
// point must not be used on a device that has been reset.
//
// Every result is reproducible bit for bit: the mode counts are integer sums,
// and the mean |k| of a bin is summed over its |k|^2 values in a fixed order.
#include <cuda_runtime.h>
#include <math.h>
#include <mutex>
#include <string.h>

#include "mgp_internal.h"

#define MGP_NA_MAX_N 1024
#define MGP_NA_MAX_BINS 2048
#define MGP_NA_BLOCKS 304
#define MGP_NA_MAX_DEV 64

// byte offsets inside the scratch array (256-byte aligned sections)
#define NA_ALIGN(x) ((((size_t)(x)) + 255) & ~(size_t)255)
#define NA_RK_MAX (3 * (MGP_NA_MAX_N / 2) * (MGP_NA_MAX_N / 2))
#define NA_OFF_RKBIN 0
#define NA_OFF_RKCNT NA_ALIGN(NA_OFF_RKBIN + sizeof(int) * (NA_RK_MAX + 1))
#define NA_OFF_BINRK NA_ALIGN(NA_OFF_RKCNT + sizeof(unsigned) * (NA_RK_MAX + 1))
#define NA_OFF_WIN NA_ALIGN(NA_OFF_BINRK + sizeof(int) * 2 * MGP_NA_MAX_BINS)
#define NA_OFF_GEON NA_ALIGN(NA_OFF_WIN + sizeof(float) * (MGP_NA_MAX_N / 2 + 1))
#define NA_OFF_GEOK NA_ALIGN(NA_OFF_GEON + sizeof(double) * MGP_NA_MAX_BINS)
#define NA_OFF_PART NA_ALIGN(NA_OFF_GEOK + sizeof(double) * MGP_NA_MAX_BINS)
#define NA_OFF_SUMS NA_ALIGN(NA_OFF_PART + sizeof(double) * MGP_NA_BLOCKS * MGP_NA_MAX_BINS)
#define NA_OFF_OUT NA_ALIGN(NA_OFF_SUMS + sizeof(double) * MGP_NA_MAX_BINS)
#define MGP_NA_SCRATCH_BYTES NA_ALIGN(NA_OFF_OUT + sizeof(double) * 3 * MGP_NA_MAX_BINS)

static __device__ __align__(256) unsigned char g_pofk_scratch[MGP_NA_SCRATCH_BYTES];

// Device address of the scratch array, looked up once per device.
static unsigned char *g_scratch_addr[MGP_NA_MAX_DEV];
static std::mutex g_scratch_mu;

static int scratch_for_current_device(unsigned char **out) {
  int dev = 0;
  MGP_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= MGP_NA_MAX_DEV) return mgp_set_error(MGP_EINVAL, "device %d out of range", dev);
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (!g_scratch_addr[dev]) {
    void *p = NULL;
    cudaError_t e = cudaGetSymbolAddress(&p, g_pofk_scratch);
    if (e != cudaSuccess || !p)
      return mgp_set_error(MGP_ECUDA, "cudaGetSymbolAddress(scratch): %s", cudaGetErrorString(e));
    g_scratch_addr[dev] = (unsigned char *)p;
  }
  *out = g_scratch_addr[dev];
  return MGP_OK;
}

// pofk_bin_index (src/compute_pofk.c:30-46) for every integer |k|^2, and the
// CIC window 1/sinc^4 per |d| (compute_pofk.c:124-148).
// Also clears the per-|k|^2 mode counts and the |k|^2 range of every bin,
// which the previous call left in the array.
__global__ void k_na_tables(int N, double kmin, double kmax, int nbins, int bintype, int *rkbin, unsigned *rkcnt,
                            int *binrk, float *win) {
  const int h = N / 2, rkmax = 3 * h * h;
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < 2 * nbins; b += gridDim.x * blockDim.x) binrk[b] = 0;
  for (int rk = blockIdx.x * blockDim.x + threadIdx.x; rk <= rkmax; rk += gridDim.x * blockDim.x) {
    rkcnt[rk] = 0u;
    double kmag = sqrt((double)rk);
    int nk;
    if (bintype == 0) nk = (int)((kmag - kmin) / (kmax - kmin) * nbins + 0.5);
    else nk = kmag <= 0.0 ? -1 : (int)(log(kmag / kmin) / log(kmax / kmin) * nbins + 0.5);
    rkbin[rk] = (nk >= 0 && nk < nbins) ? nk : -1;
    if (rk <= h) {
      double g = rk == 0 ? 1.0 : sin((M_PI * rk) / (double)N) / ((M_PI * rk) / (double)N);
      win[rk] = (float)(1.0 / (g * g * g * g));
    }
  }
}

// Weighted mode count of every integer |k|^2 with the reference's weights:
// |d0|, |d1| stand for 1 or 2 stored indices, kz = 0 and N/2 weigh 1, others
// 2 (compute_pofk.c:124-148).  The counts are integers, so the order of the
// atomic additions does not matter.  The same threads record the |k|^2
// range of every bin: rk_bin is non-decreasing in |k|^2 where it is >= 0
// (the bin index is monotone in |k|), so each bin is one contiguous range.
__global__ void k_na_geometry(int N, const int *rkbin, unsigned *rkcnt, int *binrk) {
  const int h = N / 2, rkmax = 3 * h * h;
  const long long nthr = (long long)gridDim.x * blockDim.x;
  const long long t0 = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  for (long long t = t0; t < (long long)(h + 1) * (h + 1); t += nthr) {
    int d0 = (int)(t / (h + 1)), d1 = (int)(t % (h + 1));
    unsigned m = ((d0 == 0 || d0 == h) ? 1u : 2u) * ((d1 == 0 || d1 == h) ? 1u : 2u);
    int base = d0 * d0 + d1 * d1;
    for (int d2 = 0; d2 <= h; d2++) atomicAdd(&rkcnt[base + d2 * d2], m * ((d2 == 0 || d2 == h) ? 1u : 2u));
  }
  for (long long rk = t0; rk <= rkmax; rk += nthr) {
    int b = rkbin[rk];
    if (b < 0) continue;
    if (rk == 0 || rkbin[rk - 1] != b) binrk[2 * b] = (int)rk;
    if (rk == rkmax || rkbin[rk + 1] != b) binrk[2 * b + 1] = (int)rk + 1;
  }
}

// Per bin (one warp each): mode count and sum of |k| over its |k|^2 range,
// each lane in ascending |k|^2 and the lanes combined by a fixed shuffle
// tree, so the sums do not depend on scheduling.
__global__ void k_na_binsum(int nbins, const unsigned *rkcnt, const int *binrk, double *geo_n, double *geo_k) {
  const int lane = threadIdx.x & 31;
  const int b = (int)(((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  if (b >= nbins) return;
  const int r0 = binrk[2 * b], r1 = binrk[2 * b + 1];
  double n = 0.0, k = 0.0;
  for (int rk = r0 + lane; rk < r1; rk += 32) {
    double c = (double)rkcnt[rk];
    n += c;
    k += c * sqrt((double)rk);
  }
  for (int o = 16; o > 0; o >>= 1) {
    n += __shfl_xor_sync(0xffffffffu, n, o);
    k += __shfl_xor_sync(0xffffffffu, k, o);
  }
  if (lane == 0) {
    geo_n[b] = n;
    geo_k[b] = k;
  }
}

// Normalisation and shot noise (compute_pofk.c:229-236): out = [P, kmean, n].
__global__ void k_na_finalize(int nbins, const double *sums, const double *geo_n, const double *geo_k, double norm,
                              double shot, double kunit, double *out) {
  int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nbins) return;
  double n = geo_n[b], P = 0.0, K = 0.0;
  if (n > 0) {
    P = sums[b] / n * norm - shot;
    K = geo_k[b] / n * kunit;
  }
  out[b] = P;
  out[MGP_NA_MAX_BINS + b] = K;
  out[2 * MGP_NA_MAX_BINS + b] = n;
}

extern "C" int mgp_pofk_noalloc(const float *d_deltak, int Nmesh, int Nsample, double Box, int nbins, int bintype,
                                int subtract_shotnoise, double kmin_hmpc, double kmax_hmpc, int cap, int *nbins_out,
                                double *k, double *pk, double *kmean, double *n, void *stream) {
  if (!d_deltak || !pk) return mgp_set_error(MGP_EINVAL, "null argument");
  if (Nmesh < 4 || Nmesh % 2 || Nmesh > MGP_NA_MAX_N)
    return mgp_set_error(MGP_EINVAL, "Nmesh = %d: the allocation-free P(k) supports even Nmesh <= %d", Nmesh,
                         MGP_NA_MAX_N);
  if (Nsample < 1 || !(Box > 0)) return mgp_set_error(MGP_EINVAL, "bad Nsample or Box");
  // adjust_pofk_parameters (src/compute_pofk.c:758-805), integer k units
  double kmin = kmin_hmpc * Box / (2.0 * M_PI), kmax = kmax_hmpc * Box / (2.0 * M_PI);
  if (!(bintype == 0 || bintype == 1)) bintype = 0;
  if (!(subtract_shotnoise == 0 || subtract_shotnoise == 1)) subtract_shotnoise = 1;
  if (nbins <= 0) nbins = Nmesh;
  if (kmax <= kmin) {
    kmin = bintype == 0 ? 0.0 : 1.0;
    kmax = (double)Nmesh;
  }
  if (kmin < 0.0) kmin = bintype == 0 ? 0.0 : 1.0;
  if (bintype == 1 && kmin == 0.0) kmin = 1.0;
  if (kmax > sqrt(3.0) * (double)Nmesh) kmax = (double)Nmesh;
  if (nbins > MGP_NA_MAX_BINS)
    return mgp_set_error(MGP_EINVAL, "%d bins: the allocation-free P(k) supports at most %d", nbins, MGP_NA_MAX_BINS);
  if (nbins_out) *nbins_out = nbins;
  if (cap < nbins) return mgp_set_error(MGP_EINVAL, "capacity %d < %d bins", cap, nbins);

  unsigned char *base = NULL;
  int rc = scratch_for_current_device(&base);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  int *rkbin = (int *)(base + NA_OFF_RKBIN);
  unsigned *rkcnt = (unsigned *)(base + NA_OFF_RKCNT);
  int *binrk = (int *)(base + NA_OFF_BINRK);
  float *win = (float *)(base + NA_OFF_WIN);
  double *geo_n = (double *)(base + NA_OFF_GEON), *geo_k = (double *)(base + NA_OFF_GEOK);
  double *part = (double *)(base + NA_OFF_PART), *sums = (double *)(base + NA_OFF_SUMS);
  double *out = (double *)(base + NA_OFF_OUT);
  const int h = Nmesh / 2;
  // the tables kernel clears what the previous call left in the array
  k_na_tables<<<(3 * h * h + 256) / 256, 256, 0, st>>>(Nmesh, kmin, kmax, nbins, bintype, rkbin, rkcnt, binrk, win);
  MGP_CHECK_LAUNCH();
  g_kernel_launches++;
  k_na_geometry<<<mgp_blocks_for((long long)(h + 1) * (h + 1), 8), 256, 0, st>>>(Nmesh, rkbin, rkcnt, binrk);
  MGP_CHECK_LAUNCH();
  g_kernel_launches++;
  k_na_binsum<<<(nbins * 32 + 255) / 256, 256, 0, st>>>(nbins, rkcnt, binrk, geo_n, geo_k);
  MGP_CHECK_LAUNCH();
  g_kernel_launches++;
  // the binning kernel of mgp_pofk, writing every block's partials
  int nblocks = MGP_NA_BLOCKS;
  if ((long long)nblocks * 8 > (long long)Nmesh * Nmesh) nblocks = (int)(((long long)Nmesh * Nmesh + 7) / 8);
  rc = mgp_launch_pofk(d_deltak, Nmesh, rkbin, win, nbins, part, nblocks, sums, st);
  if (rc) return rc;
  double norm = pow(Box, 3) / pow((double)Nmesh, 6);
  double shot = subtract_shotnoise ? pow(Box / (double)Nsample, 3) : 0.0;
  k_na_finalize<<<(nbins + 127) / 128, 128, 0, st>>>(nbins, sums, geo_n, geo_k, norm, shot, 2.0 * M_PI / Box, out);
  MGP_CHECK_LAUNCH();
  g_kernel_launches++;
  MGP_CUDA(cudaMemcpyAsync(pk, out, sizeof(double) * nbins, cudaMemcpyDeviceToHost, st));
  if (kmean) MGP_CUDA(cudaMemcpyAsync(kmean, out + MGP_NA_MAX_BINS, sizeof(double) * nbins, cudaMemcpyDeviceToHost, st));
  if (n) MGP_CUDA(cudaMemcpyAsync(n, out + 2 * MGP_NA_MAX_BINS, sizeof(double) * nbins, cudaMemcpyDeviceToHost, st));
  MGP_CUDA(cudaStreamSynchronize(st));
  if (k)
    for (int b = 0; b < nbins; b++)
      k[b] = (bintype == 0 ? (kmin + (kmax - kmin) / (double)nbins * b)
                           : exp(log(kmin) + log(kmax / kmin) / (double)nbins * b)) *
             2.0 * M_PI / Box;
  return MGP_OK;
}
