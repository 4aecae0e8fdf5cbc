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
// it and must be serialised by the caller.
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
#define NA_OFF_WIN NA_ALIGN(NA_OFF_RKBIN + sizeof(int) * (NA_RK_MAX + 1))
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
__global__ void k_na_tables(int N, double kmin, double kmax, int nbins, int bintype, int *rkbin, float *win) {
  const int h = N / 2, rkmax = 3 * h * h;
  for (int rk = blockIdx.x * blockDim.x + threadIdx.x; rk <= rkmax; rk += gridDim.x * blockDim.x) {
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

// Mode counts and |k| sums per bin with the reference's weights: |d0|, |d1|
// stand for 1 or 2 stored indices, kz = 0 and N/2 weigh 1, others 2.
__global__ void k_na_geometry(int N, const int *rkbin, double *geo_n, double *geo_k) {
  const int h = N / 2;
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)(h + 1) * (h + 1)) return;
  int d0 = (int)(t / (h + 1)), d1 = (int)(t % (h + 1));
  double m = ((d0 == 0 || d0 == h) ? 1.0 : 2.0) * ((d1 == 0 || d1 == h) ? 1.0 : 2.0);
  int run_bin = -1;
  double run_n = 0.0, run_k = 0.0;
  for (int d2 = 0; d2 <= h; d2++) {
    int rk = d0 * d0 + d1 * d1 + d2 * d2;
    int b = rkbin[rk];
    double w = m * ((d2 == 0 || d2 == h) ? 1.0 : 2.0);
    if (b != run_bin) {
      if (run_bin >= 0) {
        atomicAdd(&geo_n[run_bin], run_n);
        atomicAdd(&geo_k[run_bin], run_k);
      }
      run_bin = b;
      run_n = run_k = 0.0;
    }
    if (b >= 0) {
      run_n += w;
      run_k += w * sqrt((double)rk);
    }
  }
  if (run_bin >= 0) {
    atomicAdd(&geo_n[run_bin], run_n);
    atomicAdd(&geo_k[run_bin], run_k);
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
  float *win = (float *)(base + NA_OFF_WIN);
  double *geo_n = (double *)(base + NA_OFF_GEON), *geo_k = (double *)(base + NA_OFF_GEOK);
  double *part = (double *)(base + NA_OFF_PART), *sums = (double *)(base + NA_OFF_SUMS);
  double *out = (double *)(base + NA_OFF_OUT);
  const int h = Nmesh / 2;
  // the previous call's counts stay in the array: clear them
  MGP_CUDA(cudaMemsetAsync(geo_n, 0, sizeof(double) * MGP_NA_MAX_BINS, st));
  MGP_CUDA(cudaMemsetAsync(geo_k, 0, sizeof(double) * MGP_NA_MAX_BINS, st));
  k_na_tables<<<(3 * h * h + 256) / 256, 256, 0, st>>>(Nmesh, kmin, kmax, nbins, bintype, rkbin, win);
  MGP_CHECK_LAUNCH();
  long long pairs = (long long)(h + 1) * (h + 1);
  k_na_geometry<<<(int)((pairs + 255) / 256), 256, 0, st>>>(Nmesh, rkbin, geo_n, geo_k);
  MGP_CHECK_LAUNCH();
  // the binning kernel of mgp_pofk, writing every block's partials
  int nblocks = MGP_NA_BLOCKS;
  if ((long long)nblocks * 8 > (long long)Nmesh * Nmesh) nblocks = (int)(((long long)Nmesh * Nmesh + 7) / 8);
  rc = mgp_launch_pofk(d_deltak, Nmesh, rkbin, win, nbins, part, nblocks, sums, st);
  if (rc) return rc;
  double norm = pow(Box, 3) / pow((double)Nmesh, 6);
  double shot = subtract_shotnoise ? pow(Box / (double)Nsample, 3) : 0.0;
  k_na_finalize<<<(nbins + 127) / 128, 128, 0, st>>>(nbins, sums, geo_n, geo_k, norm, shot, 2.0 * M_PI / Box, out);
  MGP_CHECK_LAUNCH();
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
