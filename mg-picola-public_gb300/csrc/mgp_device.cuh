// Device helpers shared by the PM kernels and the closure kernels: the
// particle's lattice point and its cell coordinates on a mesh.
#ifndef MGP_DEVICE_CUH
#define MGP_DEVICE_CUH

// Lattice coordinates of particle p (src/main.c:257-262 ordering).
__device__ __forceinline__ void lattice_ijk(long long p, int Ns, int &i, int &j, int &k) {
  long long ns2 = (long long)Ns * Ns;
  i = (int)(p / ns2);
  long long r = p - (long long)i * ns2;
  j = (int)(r / Ns);
  k = (int)(r - (long long)j * Ns);
}

// The same for p < 2^32 in unsigned 32-bit arithmetic (a 64-bit division is
// a long instruction sequence on the GPU; the results are identical).
__device__ __forceinline__ void lattice_ijk(unsigned p, int Ns, int &i, int &j, int &k) {
  const unsigned ns = (unsigned)Ns, ns2 = ns * ns;
  const unsigned ii = p / ns2, r = p - ii * ns2, jj = r / ns;
  i = (int)ii;
  j = (int)jj;
  k = (int)(r - jj * ns);
}

// Cell index and CIC fraction along one axis for the particle at lattice
// index `li` with displacement `s` (Mpc/h) and global offset `off_cells`.
// Position in cells = li*N/Ns + s*N/Box + off; the lattice part is split into
// integer and fractional parts exactly so the small displacement keeps full
// FP32 precision.  li*N < Ns*N stays far below 2^32 for any mesh and lattice
// that fit in device memory, so the split runs in unsigned 32-bit arithmetic.
__device__ __forceinline__ void cell_frac(int li, float s, float off_cells, int N, int Ns, float scale,
                                          int &idx, float &frac) {
  const unsigned qn = (unsigned)li * (unsigned)N;
  const unsigned qi = qn / (unsigned)Ns;
  float qf = (float)(qn - qi * (unsigned)Ns) / (float)Ns;
  float w = fmaf(s, scale, off_cells) + qf;
  float fl = floorf(w);
  float fr = w - fl;
  if (fr >= 1.0f) { fr -= 1.0f; fl += 1.0f; }
  int ic = (int)qi + (int)fl;
  if (ic < 0 || ic >= N) {  // a particle more than a cell outside its lattice cell's period
    ic %= N;
    if (ic < 0) ic += N;
  }
  idx = ic;
  frac = fr;
}

// Power-of-two lattices (Ns = 2^ls, the usual set-ups): the same lattice
// coordinates and cell fractions by shifts and masks.  The results are
// identical to lattice_ijk / cell_frac: the remainder of qn / Ns is below
// 2^24, so rem * (1/Ns) is exact in FP32 as rem / Ns is.
__device__ __forceinline__ void lattice_ijk_p2(unsigned p, int ls, int &i, int &j, int &k) {
  const unsigned m = (1u << ls) - 1u;
  i = (int)(p >> (2 * ls));
  j = (int)((p >> ls) & m);
  k = (int)(p & m);
}

__device__ __forceinline__ void cell_frac_p2(int li, float s, float off_cells, int N, int ls, float inv_ns, float scale,
                                             int &idx, float &frac) {
  const unsigned qn = (unsigned)li * (unsigned)N;
  const unsigned qi = qn >> ls;
  float qf = (float)(qn & ((1u << ls) - 1u)) * inv_ns;
  float w = fmaf(s, scale, off_cells) + qf;
  float fl = floorf(w);
  float fr = w - fl;
  if (fr >= 1.0f) { fr -= 1.0f; fl += 1.0f; }
  int ic = (int)qi + (int)fl;
  if (ic < 0 || ic >= N) {
    ic %= N;
    if (ic < 0) ic += N;
  }
  idx = ic;
  frac = fr;
}

// log2(Ns) when Ns is a power of two, else -1 (host and device).
__host__ __device__ __forceinline__ int lattice_log2(int Ns) {
  if (Ns <= 0 || (Ns & (Ns - 1))) return -1;
  int l = 0;
  while ((1 << l) < Ns) l++;
  return l;
}


// Fourier-space filter of the fifth-force solvers per integer |k|^2 = rk
// (grid units): kind 1 SmoothDensityField (src/mg.h:268-309) with the
// smoothing filters of src/mg.h:318-338 (Gaussian, top-hat, sharp-k), kR =
// sqrt(rk) kR1, times norm; kind 2 the inverse Laplacian of DivideByLaplacian
// (src/mg.h:21-64), -norm / rk (0 at k = 0).  filter takes the
// MGP_FILTER_* values (1 Gaussian, 2 top-hat, 3 sharp-k).
__device__ __forceinline__ float mg_kfilter(int rk, int kind, int filter, float kR1, float norm) {
  if (kind == 2) return rk == 0 ? 0.0f : -norm / (float)rk;
  float kR = sqrtf((float)rk) * kR1, f = 1.0f;
  if (filter == 1) f = expf(-0.5f * kR * kR);
  else if (filter == 2) f = kR < 1e-5f ? 1.0f : 3.0f / (kR * kR * kR) * (sinf(kR) - kR * cosf(kR));
  else if (filter == 3) f = kR < 1.0f ? 1.0f : 0.0f;
  return f * norm;
}

#endif
