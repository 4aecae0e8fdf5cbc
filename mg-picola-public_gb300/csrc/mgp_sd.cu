// Scale-dependent growth on the device (the SCALEDEPENDENT build of the
// reference): per-step LPT displacement fields from the stored delta(k) and
// 2LPT source S(k) of the IC, scaled by growth factors D(k, a) of the 2D
// growth tables (src/2LPT.c:1539-2005, src/cosmo.c:798-1010).
//
// The reference builds each field per LPT order on the full mesh: multiply
// by i k/k^2 G(k, a), three N^3 C2R transforms, trilinear read-out at the
// Lagrangian lattice, mean removal (from_cdisp_store_to_ZA).  Every reader
// of the fields adds the two orders, and when Nmesh = r Nsample the lattice
// points are mesh points (the trilinear weights are 1 and 0), so here:
//   - both orders are combined in k space: S(k) = T1(|k|^2) delta(k) +
//     T2(|k|^2) (-S2(k)), with T per integer |k|^2 from one table kernel;
//   - sampling every r-th mesh point of the C2R equals an Ns^3 C2R of the
//     spectrum folded onto the Ns grid, G(k') = sum over the r^3 aliases
//     k = k' + Ns a of the full (Hermitian-extended) spectrum, so each field
//     costs one fold pass over the N^3 spectrum and three Ns^3 C2R instead of
//     three N^3 C2R per order;
//   - the mean over the lattice is G(0), so mean removal is G(0) = 0.
// When Nmesh is not a multiple of Nsample the lattice points fall between mesh
// points, and the fields follow the reference's algorithm itself: per
// component the full-mesh spectrum (k_sd_full), an N^3 C2R, the trilinear
// read-out at the lattice points (k_sd_readout, src/2LPT.c:1642-1704) and the
// removal of the lattice mean (src/2LPT.c:1714-1728).
// On the kz = 0 and kz = N/2 planes the C2R keeps only the Hermitian part of
// its input (FFTW's half-complex semantics); with Hermitian delta and S2
// that zeroes the derivative components whose own index is the Nyquist one,
// as in the force kernel.
#include <cuda_runtime.h>
#include <cufft.h>
#include <math.h>
#include <string.h>

#include <vector>

#include "mgp_internal.h"

namespace {

constexpr int kThreads = 256;
// blocks of the general-ratio read-out (fixed, so its mean sums in a fixed order)
#define SD_READOUT_BLOCKS 1216

// Integer wave number of index idx (src/2LPT.c:1586-1602): idx < N/2 -> idx,
// else idx - N, so N/2 maps to -N/2.
__device__ __forceinline__ int sd_d(int idx, int N) { return idx < N / 2 ? idx : idx - N; }

struct SdRecipe {
  // output o of the float4 table: coef * (C[num] - C[sub]) / C[nrm]
  // (sub < 0: no subtraction), times kfac / |k|^2
  int num[4], sub[4], nrm[4];
  double coef[4];
  int nout;
  int ny;          // nodes per column
  double y0, dy;   // ln k of node 0 and spacing
  double kfac;     // 2 pi / Box (h/Mpc per integer wave number)
};

// Cubic Hermite in ln k of one growth-table column (values then d/d ln k at
// the ny nodes), ln k clamped to the table range as Lookup_GSL_2D_Spline.
__device__ double column_at(const double *__restrict__ col, int ny, double y0, double dy, double y) {
  double t = (y - y0) / dy;
  if (t < 0.0) t = 0.0;
  if (t > (double)(ny - 1)) t = (double)(ny - 1);
  int j = (int)t;
  if (j > ny - 2) j = ny - 2;
  double u = t - (double)j;
  const double *dv = col + ny;
  return (1 + 2 * u) * (1 - u) * (1 - u) * col[j] + u * u * (3 - 2 * u) * col[j + 1] +
         u * (1 - u) * (1 - u) * dy * dv[j] + u * u * (u - 1) * dy * dv[j + 1];
}

__global__ void k_sd_table(const double *__restrict__ cols, SdRecipe r, long long nmax, float4 *__restrict__ tab) {
  long long stride = (long long)gridDim.x * blockDim.x;
  for (long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x; n <= nmax; n += stride) {
    float o[4] = {0.f, 0.f, 0.f, 0.f};
    if (n > 0) {
      double kmag = sqrt((double)n) * r.kfac, y = log(kmag), inv = r.kfac / (kmag * kmag);
      const long long cs = 2LL * r.ny;
      for (int q = 0; q < r.nout; q++) {
        double g = column_at(cols + r.num[q] * cs, r.ny, r.y0, r.dy, y);
        if (r.sub[q] >= 0) g -= column_at(cols + r.sub[q] * cs, r.ny, r.y0, r.dy, y);
        g /= column_at(cols + r.nrm[q] * cs, r.ny, r.y0, r.dy, y);
        o[q] = (float)(r.coef[q] * g * inv);
      }
    }
    tab[n] = make_float4(o[0], o[1], o[2], o[3]);
  }
}

// One thread per output mode k' of the Ns half-complex grid; sums the r^3
// aliases of the full spectrum F_a(k) = i d_a T(|k|^2) . (delta, -S2) for one
// or two fields (table components xy -> field 0, zw -> field 1).
__global__ void __launch_bounds__(kThreads) k_sd_fold(const float2 *__restrict__ d1, const float2 *__restrict__ d2,
                                                       const float4 *__restrict__ tab, int N, int Ns, int r,
                                                       int nfields, float2 *__restrict__ out0,
                                                       float2 *__restrict__ out1, long long ostride) {
  const int NH = N / 2 + 1, NHs = Ns / 2 + 1;
  // one warp per folded (kx, ky) row, lanes along kz: no division per mode
  const int lane = threadIdx.x & 31;
  const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
  for (long long row = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; row < (long long)Ns * Ns; row += nw)
  for (int kzp = lane; kzp < NHs; kzp += 32) {
    const long long o = row * NHs + kzp;
    const int kxp = (int)(row / Ns), kyp = (int)(row - (long long)kxp * Ns);
    float2 G[2][3];
#pragma unroll
    for (int f = 0; f < 2; f++)
#pragma unroll
      for (int a = 0; a < 3; a++) G[f][a] = make_float2(0.f, 0.f);
    if (o != 0) {
      for (int ax = 0; ax < r; ax++) {
        const int kx = kxp + Ns * ax;
        for (int ay = 0; ay < r; ay++) {
          const int ky = kyp + Ns * ay;
          for (int az = 0; az < r; az++) {
            const int kz = kzp + Ns * az;
            // stored half space, or the conjugate of the mirrored mode
            const bool cj = 2 * kz > N;
            const int sx = cj ? (kx == 0 ? 0 : N - kx) : kx, sy = cj ? (ky == 0 ? 0 : N - ky) : ky, sz = cj ? N - kz : kz;
            const long long c = ((long long)sx * N + sy) * NH + sz;
            const int dx = sd_d(sx, N), dy = sd_d(sy, N), dz = sd_d(sz, N);
            const float4 t = __ldg(tab + ((long long)dx * dx + (long long)dy * dy + (long long)dz * dz));
            const float2 u = __ldg(d1 + c), w = __ldg(d2 + c);
            float m[3] = {(float)dx, (float)dy, (float)dz};
            if (sz == 0 || 2 * sz == N) {
              if (2 * sx == N) m[0] = 0.f;
              if (2 * sy == N) m[1] = 0.f;
              m[2] = 0.f;
            }
            const float sg = cj ? -1.f : 1.f;
            float2 S0 = make_float2(t.x * u.x + t.y * w.x, t.x * u.y + t.y * w.y);
#pragma unroll
            for (int a = 0; a < 3; a++) {
              G[0][a].x -= m[a] * S0.y;
              G[0][a].y += sg * m[a] * S0.x;
            }
            if (nfields > 1) {
              float2 S1 = make_float2(t.z * u.x + t.w * w.x, t.z * u.y + t.w * w.y);
#pragma unroll
              for (int a = 0; a < 3; a++) {
                G[1][a].x -= m[a] * S1.y;
                G[1][a].y += sg * m[a] * S1.x;
              }
            }
          }
        }
      }
    }
#pragma unroll
    for (int a = 0; a < 3; a++) out0[a * ostride + o] = G[0][a];
    if (nfields > 1) {
#pragma unroll
      for (int a = 0; a < 3; a++) out1[a * ostride + o] = G[1][a];
    }
  }
}

// Full-mesh spectrum of component a of field f (table components xy for
// f = 0, zw for f = 1): i d_a T(|k|^2) . (delta, -S2), one warp per (kx, ky)
// row (from_cdisp_store_to_ZA, src/2LPT.c:1586-1627), with the Nyquist
// derivative entries written as zero as in k_sd_fold.
__global__ void __launch_bounds__(kThreads) k_sd_full(const float2 *__restrict__ d1, const float2 *__restrict__ d2,
                                                       const float4 *__restrict__ tab, int N, int f, int a,
                                                       float2 *__restrict__ out) {
  const int NH = N / 2 + 1;
  const int lane = threadIdx.x & 31;
  const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
  for (long long row = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; row < (long long)N * N; row += nw) {
    const int kx = (int)(row / N), ky = (int)(row - (long long)kx * N);
    const int dx = sd_d(kx, N), dy = sd_d(ky, N);
    for (int kz = lane; kz < NH; kz += 32) {
      const long long c = row * NH + kz;
      const int dz = sd_d(kz, N);
      const float4 t = __ldg(tab + ((long long)dx * dx + (long long)dy * dy + (long long)dz * dz));
      const float T1 = f == 0 ? t.x : t.z, T2 = f == 0 ? t.y : t.w;
      const float2 u = __ldg(d1 + c), w = __ldg(d2 + c);
      const float2 S = make_float2(T1 * u.x + T2 * w.x, T1 * u.y + T2 * w.y);
      float m = a == 0 ? (float)dx : (a == 1 ? (float)dy : (float)dz);
      if (kz == 0 || 2 * kz == N) {
        if ((a == 0 && 2 * kx == N) || (a == 1 && 2 * ky == N) || a == 2) m = 0.f;
      }
      out[c] = make_float2(-m * S.y, m * S.x);
    }
  }
}

// Trilinear read-out of the real field at the Lagrangian lattice points
// (i, j, k) N/Ns (src/2LPT.c:1642-1704): fractions from the exact integer
// split of i N / Ns, periodic neighbours; per-block sums of the values for
// the mean (fixed order, FP64).
__global__ void __launch_bounds__(kThreads) k_sd_readout(const float *__restrict__ g, int N, int Ns, long long np,
                                                          float *__restrict__ out, int pitch,
                                                          double *__restrict__ partials) {
  __shared__ double sh[kThreads / 32];
  const long long P = 2 * (long long)(N / 2 + 1);
  double acc = 0.0;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < np; p += stride) {
    const long long ij = p / Ns;
    const int k = (int)(p - ij * Ns), i = (int)(ij / Ns), j = (int)(ij - (long long)i * Ns);
    int idx[3], nxt[3];
    float fr[3];
    const int l[3] = {i, j, k};
#pragma unroll
    for (int q = 0; q < 3; q++) {
      const long long qn = (long long)l[q] * N;
      idx[q] = (int)(qn / Ns);
      fr[q] = (float)(qn - (long long)idx[q] * Ns) / (float)Ns;
      nxt[q] = idx[q] + 1 >= N ? idx[q] + 1 - N : idx[q] + 1;
    }
    const float u = fr[0], v = fr[1], w = fr[2];
    const long long r00 = ((long long)idx[0] * N + idx[1]) * P, r01 = ((long long)idx[0] * N + nxt[1]) * P;
    const long long r10 = ((long long)nxt[0] * N + idx[1]) * P, r11 = ((long long)nxt[0] * N + nxt[1]) * P;
    const float val = g[r00 + idx[2]] * (1 - u) * (1 - v) * (1 - w) + g[r00 + nxt[2]] * (1 - u) * (1 - v) * w +
                      g[r01 + idx[2]] * (1 - u) * v * (1 - w) + g[r01 + nxt[2]] * (1 - u) * v * w +
                      g[r10 + idx[2]] * u * (1 - v) * (1 - w) + g[r10 + nxt[2]] * u * (1 - v) * w +
                      g[r11 + idx[2]] * u * v * (1 - w) + g[r11 + nxt[2]] * u * v * w;
    out[ij * pitch + k] = val;
    acc += (double)val;
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); q++) t += sh[q];
    partials[blockIdx.x] = t;
  }
}

// Removes the lattice mean (src/2LPT.c:1714-1728): every block sums the
// read-out partials in the same fixed order, then subtracts.
__global__ void k_sd_sub_mean(float *__restrict__ out, int pitch, int Ns, long long np,
                              const double *__restrict__ partials, int nparts) {
  __shared__ float mean;
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int q = 0; q < nparts; q++) t += partials[q];
    mean = (float)(t / (double)np);
  }
  __syncthreads();
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < np; p += stride) {
    const long long ij = p / Ns;
    out[ij * pitch + (p - ij * Ns)] -= mean;
  }
}

// IC particle state (src/main.c:256-307, SCALEDEPENDENT branch): the
// displacement from the lattice is the D field (1LPT + 2LPT, already at a_i);
// the velocity is 0 for COLA, else the dDdy field.
__global__ void k_sd_init_state(const float *__restrict__ Dslot, const float *__restrict__ Vslot, long long gsz,
                                int pitch, long long np, int Ns, int cola, float *__restrict__ s,
                                float *__restrict__ v) {
  long long stride = (long long)gridDim.x * blockDim.x;
  const long long ns2 = (long long)Ns * Ns;
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < np; p += stride) {
    const long long row = p / Ns, k = p - row * Ns;
    const long long od = row * pitch + k;
    (void)ns2;
#pragma unroll
    for (int a = 0; a < 3; a++) {
      s[a * np + p] = Dslot[a * gsz + od];
      v[a * np + p] = cola ? 0.0f : Vslot[a * gsz + od];
    }
  }
}

// -X: complex copy with sign (the stored 2LPT source is -S2, zero at k = 0)
__global__ void k_sd_store(const float2 *__restrict__ dk, const float2 *__restrict__ src, long long n,
                           float2 *__restrict__ o1, float2 *__restrict__ o2) {
  long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    o1[i] = dk[i];
    float2 s = src[i];
    o2[i] = i == 0 ? make_float2(0.f, 0.f) : make_float2(-s.x, -s.y);
  }
}

}  // namespace

int mgp_sd_alloc(mgp_ctx *c) {
  const int N = c->g.N, Ns = c->Ns;
  if (Ns % 2) return mgp_set_error(MGP_EINVAL, "scale-dependent growth needs an even Nsample (%d)", Ns);
  c->sd = 1;
  // alias fold when the lattice points are mesh points, else the full-mesh
  // path with the trilinear read-out (0)
  c->sd_fold = N % Ns == 0 ? N / Ns : 0;
  if (!c->sd_fold) {
    MGP_CUDA(cudaMalloc(&c->sd_full, sizeof(float) * (size_t)c->g.nreal));
    MGP_CUDA(cudaMalloc(&c->sd_part, sizeof(double) * SD_READOUT_BLOCKS));
  }
  c->sd_pitch = 2 * (Ns / 2 + 1);
  c->sd_grid = (long long)Ns * Ns * c->sd_pitch;
  c->sd_nmax = 3LL * (N / 2) * (N / 2);
  for (int q = 0; q < 3; q++) {
    c->sd_kind[q] = -1;
    c->sd_a[q] = c->sd_aff[q] = 0.0;
  }
  for (int q = 0; q < 2; q++) MGP_CUDA(cudaMalloc(&c->sd_dk[q], sizeof(float) * 2 * (size_t)c->g.ncomplex));
  for (int q = 0; q < 3; q++) {
    MGP_CUDA(cudaMalloc(&c->sd_slot[q], sizeof(float) * 3 * (size_t)c->sd_grid));
    MGP_CUDA(cudaMemset(c->sd_slot[q], 0, sizeof(float) * 3 * (size_t)c->sd_grid));
  }
  const int ny = c->cosmo.sd_tab[0].ny;
  MGP_CUDA(cudaMalloc(&c->sd_cols, sizeof(double) * 2 * ny * 10));
  MGP_CUDA(cudaMalloc(&c->sd_tab, sizeof(float) * 4 * (size_t)(c->sd_nmax + 1)));
  long long n[3] = {Ns, Ns, Ns};
  long long rembed[3] = {Ns, Ns, c->sd_pitch};
  long long cembed[3] = {Ns, Ns, Ns / 2 + 1};
  size_t ws = 0;
  MGP_CUFFT(cufftCreate(&c->plan_c2r_s));
  MGP_CUFFT(cufftSetAutoAllocation(c->plan_c2r_s, 0));
  MGP_CUFFT(cufftMakePlanMany64(c->plan_c2r_s, 3, n, cembed, 1, (long long)Ns * Ns * (Ns / 2 + 1), rembed, 1,
                                c->sd_grid, CUFFT_C2R, 1, &ws));
  if (ws > c->fft_work_bytes)
    return mgp_set_error(MGP_ECUFFT, "Nsample^3 C2R needs %zu bytes of work area, more than the mesh plans' %zu",
                         ws, c->fft_work_bytes);
  MGP_CUFFT(cufftSetWorkArea(c->plan_c2r_s, c->fft_work));
  MGP_CUFFT(cufftSetStream(c->plan_c2r_s, c->stream));
  return MGP_OK;
}

void mgp_sd_free(mgp_ctx *c) {
  if (!c->sd) return;
  for (int q = 0; q < 2; q++)
    if (c->sd_dk[q]) cudaFree(c->sd_dk[q]);
  for (int q = 0; q < 3; q++)
    if (c->sd_slot[q]) cudaFree(c->sd_slot[q]);
  if (c->sd_cols) cudaFree(c->sd_cols);
  if (c->sd_tab) cudaFree(c->sd_tab);
  if (c->sd_full) cudaFree(c->sd_full);
  if (c->sd_part) cudaFree(c->sd_part);
  cufftDestroy(c->plan_c2r_s);
  c->sd = 0;
}

int mgp_sd_store(mgp_ctx *c, const float *deltak, const float *source2k) {
  const long long n = c->g.ncomplex;
  k_sd_store<<<mgp_blocks_for(n, 8), kThreads, 0, c->stream>>>((const float2 *)deltak, (const float2 *)source2k, n,
                                                              (float2 *)c->sd_dk[0], (float2 *)c->sd_dk[1]);
  MGP_CHECK_LAUNCH();
  g_kernel_launches++;
  return MGP_OK;
}

// slot of each field type (the reference's P[] members, src/2LPT.c:1815-1829)
static int slot_of(int type) {
  switch (type) {
    case MGP_FIELD_D:
    case MGP_FIELD_ddDddy: return 0;
    case MGP_FIELD_deltaD: return 1;
    case MGP_FIELD_dDdy: return 2;
    default: return -1;
  }
}

// One fold + C2R pass for up to two fields.
static int fields_pass(mgp_ctx *c, double A, double AFF, int n, const int *types) {
  const mgp_bicubic *tb = &c->cosmo.sd_tab[0];
  const int ny = tb->ny;
  const double nmesh3 = (double)c->g.N * (double)c->g.N * (double)c->g.N;
  // columns: 0 D(a=1), 1 D2(a=1), then per field the needed ones
  std::vector<double> cols((size_t)2 * ny * 10);
  int ncol = 0;
  auto add = [&](int which, double a) {
    mgp_cosmo_sd_column(&c->cosmo, which, a, &cols[(size_t)ncol * 2 * ny], &cols[(size_t)ncol * 2 * ny + ny]);
    return ncol++;
  };
  const int n1 = add(0, 1.0), n2 = add(3, 1.0);
  SdRecipe r;
  memset(&r, 0, sizeof(r));
  r.nout = 2 * n;
  r.ny = ny;
  r.y0 = tb->y[0];
  r.dy = (tb->y[ny - 1] - tb->y[0]) / (double)(ny - 1);
  r.kfac = 2.0 * M_PI / c->p.Box;
  for (int f = 0; f < n; f++) {
    // order 1 (normfactor 1) and order 2 (normfactor -3/7/N^3), 2LPT.c:1547-1557
    for (int o = 0; o < 2; o++) {
      const int q = 2 * f + o, base = o == 0 ? 0 : 3;
      r.nrm[q] = o == 0 ? n1 : n2;
      r.coef[q] = o == 0 ? 1.0 : -3.0 / 7.0 / nmesh3;
      r.sub[q] = -1;
      switch (types[f]) {
        case MGP_FIELD_D: r.num[q] = add(base, A); break;
        case MGP_FIELD_dDdy: r.num[q] = add(base + 1, A); break;
        case MGP_FIELD_ddDddy: r.num[q] = add(base + 2, A); break;
        case MGP_FIELD_deltaD:
          r.num[q] = add(base, AFF);
          r.sub[q] = add(base, A);
          break;
      }
    }
  }
  MGP_CUDA(cudaMemcpyAsync(c->sd_cols, cols.data(), sizeof(double) * 2 * ny * ncol, cudaMemcpyHostToDevice,
                           c->stream));
  k_sd_table<<<mgp_blocks_for(c->sd_nmax + 1, 8), kThreads, 0, c->stream>>>(c->sd_cols, r, c->sd_nmax,
                                                                            (float4 *)c->sd_tab);
  MGP_CHECK_LAUNCH();
  g_kernel_launches++;
  const int Ns = c->Ns;
  if (!c->sd_fold) {
    // Nmesh not a multiple of Nsample: per field and component the
    // full-mesh spectrum, an N^3 C2R, the trilinear read-out and the mean
    const int N = c->g.N;
    for (int f = 0; f < n; f++) {
      const int s = slot_of(types[f]);
      for (int a = 0; a < 3; a++) {
        k_sd_full<<<mgp_blocks_for((long long)N * N * 32, 8), kThreads, 0, c->stream>>>(
            (const float2 *)c->sd_dk[0], (const float2 *)c->sd_dk[1], (const float4 *)c->sd_tab, N, f, a,
            (float2 *)c->sd_full);
        MGP_CHECK_LAUNCH();
        g_kernel_launches++;
        MGP_CUFFT(cufftExecC2R(c->plan_c2r_1, (cufftComplex *)c->sd_full, (cufftReal *)c->sd_full));
        float *out = c->sd_slot[s] + a * c->sd_grid;
        k_sd_readout<<<SD_READOUT_BLOCKS, kThreads, 0, c->stream>>>(c->sd_full, N, Ns, c->np, out, c->sd_pitch,
                                                                    c->sd_part);
        MGP_CHECK_LAUNCH();
        g_kernel_launches++;
        k_sd_sub_mean<<<SD_READOUT_BLOCKS, kThreads, 0, c->stream>>>(out, c->sd_pitch, Ns, c->np, c->sd_part,
                                                                     SD_READOUT_BLOCKS);
        MGP_CHECK_LAUNCH();
        g_kernel_launches++;
      }
      c->sd_kind[s] = types[f];
      c->sd_a[s] = A;
      c->sd_aff[s] = AFF;
    }
    return MGP_OK;
  }
  float *o0 = c->sd_slot[slot_of(types[0])], *o1 = n > 1 ? c->sd_slot[slot_of(types[1])] : NULL;
  k_sd_fold<<<mgp_blocks_for((long long)Ns * Ns * 32, 8), kThreads, 0, c->stream>>>(
      (const float2 *)c->sd_dk[0], (const float2 *)c->sd_dk[1], (const float4 *)c->sd_tab, c->g.N, Ns, c->sd_fold, n,
      (float2 *)o0, (float2 *)o1, c->sd_grid / 2);
  MGP_CHECK_LAUNCH();
  g_kernel_launches++;
  for (int f = 0; f < n; f++) {
    float *base = c->sd_slot[slot_of(types[f])];
    for (int a = 0; a < 3; a++) {
      float *g = base + a * c->sd_grid;
      MGP_CUFFT(cufftExecC2R(c->plan_c2r_s, (cufftComplex *)g, (cufftReal *)g));
    }
    const int s = slot_of(types[f]);
    c->sd_kind[s] = types[f];
    c->sd_a[s] = A;
    c->sd_aff[s] = AFF;
  }
  return MGP_OK;
}

int mgp_sd_fields(mgp_ctx *c, double A, double AFF, int n, const int *types) {
  if (!c->sd) return mgp_set_error(MGP_ESTATE, "the context was not created with scaledependent = 1");
  if (n < 1 || n > 3 || !types) return mgp_set_error(MGP_EINVAL, "1 to 3 field types expected (got %d)", n);
  int used[3] = {0, 0, 0};
  for (int f = 0; f < n; f++) {
    int s = slot_of(types[f]);
    if (s < 0) return mgp_set_error(MGP_EINVAL, "unknown field type %d", types[f]);
    if (used[s]) return mgp_set_error(MGP_EINVAL, "field types %d share one particle slot", types[f]);
    used[s] = 1;
  }
  if (!(A > 0) || (!(AFF > 0) && n > 0)) return mgp_set_error(MGP_EINVAL, "scale factors must be positive");
  int rc = fields_pass(c, A, AFF, n > 2 ? 2 : n, types);
  if (rc == MGP_OK && n > 2) rc = fields_pass(c, A, AFF, 1, types + 2);
  return rc;
}

int mgp_sd_init_particles(mgp_ctx *c) {
  k_sd_init_state<<<mgp_blocks_for(c->np, 8), kThreads, 0, c->stream>>>(c->sd_slot[0], c->sd_slot[2], c->sd_grid,
                                                                        c->sd_pitch, c->np, c->Ns, c->p.UseCOLA != 0,
                                                                        c->s, c->v);
  MGP_CHECK_LAUNCH();
  g_kernel_launches++;
  return MGP_OK;
}

extern "C" int mgp_assign_displacement_fields(mgp_ctx *c, double A, double AFF, int n, const int *types) {
  if (!c) return mgp_set_error(MGP_EINVAL, "null context");
  MGP_CUDA(cudaSetDevice(c->device));
  int rc = mgp_sd_fields(c, A, AFF, n, types);
  if (rc) return rc;
  MGP_CUDA(cudaStreamSynchronize(c->stream));
  return MGP_OK;
}
