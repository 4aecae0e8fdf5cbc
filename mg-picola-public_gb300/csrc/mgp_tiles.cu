// Cell-tile order of the particles for the two particle passes of the PM
// step (sm_103a).
//
// The IC writes the particles in Lagrangian (lattice) order.  Once per step,
// before the deposit, the particles are counted and bucketed by the
// TX x TX x TZ-cell tile of their CIC base cell (a counting sort of the
// particle indices):
//   k_tile_key      tile of every particle, tile counts (warp-aggregated)
//   k_scan_*        exclusive prefix sum of the counts = tile offsets
//   k_tile_scatter  particle indices bucketed by tile and, for a single box,
//                   the lattice point of every slot beside its index
// Then
//   k_cic_tiles_own PtoMesh (src/auxPM.c:280-357) for a single box: one block
//   + k_cic_halo    per tile accumulates its particles' CIC weights in a
//                   shared-memory copy of the tile plus its +1 halo, stores
//                   the tile's interior cells itself (no pre-set mesh) and
//                   leaves the halo as float2 pairs, which the second pass
//                   adds to the neighbouring tiles' cells;
//   k_cic_tiles     the same sums for batches, added to a mesh pre-set to -1
//                   with one vector reduction per pair of cells;
//   k_ikd_tiles     MtoParticles + Kick + Drift (src/auxPM.c:560-644,
//                   src/main.c:688-787) per tile: the block copies the three
//                   force grids over the tile and its +1 halo into shared
//                   memory, interpolates its particles' forces there, and
//                   writes every particle's s and v to its slot in the tile
//                   order (the sort's lattice map then describes the arrays),
//                   so that the arrays follow the particles and the next
//                   step's reads stay nearly sequential.
// Any order gives the same density and forces (up to the order of
// floating-point sums); the tile order restores the locality that the
// Lagrangian order loses as the particles cluster.
//
// A batch of B boxes (particle arrays 3 np floats apart, meshes one real
// grid apart) sorts and deposits all boxes in the same launches: box b's
// tiles follow those of boxes 0..b-1 and the order holds the global index
// b np + p.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include "mgp_device.cuh"
#include "mgp_internal.h"

namespace {

constexpr int kThreads = 256;
constexpr int kScanItems = 16;                     // per thread in a scan block
constexpr int kScanChunk = kThreads * kScanItems;  // elements per scan block

// CIC base cell and fractions of a particle with displacement (sx, sy, sz)
// at lattice point lat (the same arithmetic as k_cic and the kick).
template <bool P2>
__device__ __forceinline__ void cell_of(float sx, float sy, float sz, unsigned lat, int Ns, int ls, float inv_ns, int N,
                                        float scale, float ox, float oy, float oz, int &ix, int &iy, int &iz,
                                        float &DX, float &DY, float &DZ) {
  int i, j, k;
  if (P2) {
    lattice_ijk_p2(lat, ls, i, j, k);
    cell_frac_p2(i, sx, ox, N, ls, inv_ns, scale, ix, DX);
    cell_frac_p2(j, sy, oy, N, ls, inv_ns, scale, iy, DY);
    cell_frac_p2(k, sz, oz, N, ls, inv_ns, scale, iz, DZ);
  } else {
    lattice_ijk(lat, Ns, i, j, k);
    cell_frac(i, sx, ox, N, Ns, scale, ix, DX);
    cell_frac(j, sy, oy, N, Ns, scale, iy, DY);
    cell_frac(k, sz, oz, N, Ns, scale, iz, DZ);
  }
}

// The same for the particle in array slot p.
template <bool P2>
__device__ __forceinline__ void particle_cell(const float *__restrict__ s, long long np, long long p, unsigned lat,
                                              int Ns, int ls, float inv_ns, int N, float scale, float ox, float oy,
                                              float oz, int &ix, int &iy, int &iz, float &DX, float &DY, float &DZ) {
  cell_of<P2>(s[p], s[np + p], s[2 * np + p], lat, Ns, ls, inv_ns, N, scale, ox, oy, oz, ix, iy, iz, DX, DY, DZ);
}

// Tile shapes: T = 8 and 16 are cubic tiles of T^3 cells; T = 64 (kElong)
// is 8 x 8 x 64 cells, whose rows of 64 cells (256 bytes) make the deposit's
// flush and the kick's force staging move long contiguous pieces.
constexpr int kElong = 64;
__host__ __device__ constexpr int tile_tx(int T) { return T == kElong ? 8 : T; }

// The L-th tile of a kernel's sweep over an ntx x ntx x ntz tile grid: with
// ntx and ntz multiples of 8 the tiles go in blocks of 8^3 tiles (the
// blocks, and the tiles inside one, in x, y, z order), so that the tiles in
// flight at one time are neighbours and the grid lines and particles they
// share are found in L2; else in index order.
__device__ __forceinline__ int tile_at(int L, int ntx, int ntz) {
  if ((ntx & 7) || (ntz & 7)) return L;
  const int gx = ntx >> 3, gz = ntz >> 3, sup = L >> 9, w = L & 511;
  const int sx = sup / (gx * gz), sy = (sup / gz) % gx, sz = sup % gz;
  const int tx = (sx << 3) + (w >> 6), ty = (sy << 3) + ((w >> 3) & 7), tz = (sz << 3) + (w & 7);
  return (tx * ntx + ty) * ntz + tz;
}

// Asynchronous 16-byte global -> shared copies (cp.async, cached in L2
// only): both addresses 16-byte aligned.
__device__ __forceinline__ unsigned smem_u32(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void cp_async16(float *dst, const float *src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// Tile of every particle and the per-tile counts.  The loop runs in whole
// warps (warp-aligned starts, stride a multiple of 32) so that the lanes of
// a warp can merge their count increments per tile.
template <bool P2>
__global__ void __launch_bounds__(kThreads) k_tile_key(const float *__restrict__ s, const mgp_dstate *__restrict__ st,
                                                       long long np, int Ns, int ls, int N, float scale, int sx,
                                                       int sz, int ntx, int ntz, const unsigned *__restrict__ q,
                                                       unsigned *__restrict__ tile_of,
                                                       unsigned *__restrict__ count) {
  // box blockIdx.y of a batch: particles 3 np apart, its tiles after those
  // of the boxes before it, tile_of indexed by the particle's global index
  const unsigned box = blockIdx.y, ntiles = (unsigned)ntx * ntx * ntz;
  s += (long long)box * 3 * np;
  st += box;
  tile_of += (long long)box * np;
  const float ox = (float)(st->cx[0] * scale), oy = (float)(st->cx[1] * scale), oz = (float)(st->cx[2] * scale);
  const float inv_ns = 1.0f / (float)Ns;
  const int lane = threadIdx.x & 31;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long base = (long long)blockIdx.x * blockDim.x + (threadIdx.x & ~31); base < np; base += stride) {
    const long long p = base + lane;
    const bool on = p < np;
    const unsigned am = __ballot_sync(0xffffffffu, on);
    if (!on) continue;
    int ix, iy, iz;
    float DX, DY, DZ;
    particle_cell<P2>(s, np, p, q ? q[p] : (unsigned)p, Ns, ls, inv_ns, N, scale, ox, oy, oz, ix, iy, iz, DX, DY,
                      DZ);
    const unsigned t = box * ntiles + ((unsigned)(ix >> sx) * (unsigned)ntx + (unsigned)(iy >> sx)) * (unsigned)ntz +
                       (unsigned)(iz >> sz);
    tile_of[p] = t;
    const unsigned same = __match_any_sync(am, t);
    if (lane == __ffs(same) - 1) atomicAdd(count + t, (unsigned)__popc(same));
  }
}

// Exclusive scan of n counts: per block of kScanChunk a local scan and its
// total, a one-block scan of the totals, then the block offsets added.
__device__ __forceinline__ unsigned block_excl_scan(unsigned v, unsigned *sh, unsigned &total) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  unsigned x = v;
  for (int o = 1; o < 32; o <<= 1) {
    unsigned y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) sh[w] = x;
  __syncthreads();
  if (w == 0) {
    unsigned y = lane < (int)(blockDim.x >> 5) ? sh[lane] : 0u;
    for (int o = 1; o < 32; o <<= 1) {
      unsigned z = __shfl_up_sync(0xffffffffu, y, o);
      if (lane >= o) y += z;
    }
    sh[lane] = y;
  }
  __syncthreads();
  total = sh[(blockDim.x >> 5) - 1];
  const unsigned res = x - v + (w > 0 ? sh[w - 1] : 0u);
  __syncthreads();
  return res;
}

__global__ void __launch_bounds__(kThreads) k_scan_local(const unsigned *__restrict__ in, long long n,
                                                         unsigned *__restrict__ out, unsigned *__restrict__ bsum) {
  __shared__ unsigned sh[32];
  const long long b0 = (long long)blockIdx.x * kScanChunk + (long long)threadIdx.x * kScanItems;
  unsigned v[kScanItems], acc = 0;
#pragma unroll
  for (int q = 0; q < kScanItems; q++) {
    v[q] = b0 + q < n ? in[b0 + q] : 0u;
    acc += v[q];
  }
  unsigned total;
  unsigned off = block_excl_scan(acc, sh, total);
#pragma unroll
  for (int q = 0; q < kScanItems; q++) {
    if (b0 + q < n) out[b0 + q] = off;
    off += v[q];
  }
  if (threadIdx.x == 0) bsum[blockIdx.x] = total;
}

// One block: exclusive scan of the nb block totals in place (nb <= kScanChunk).
__global__ void __launch_bounds__(kThreads) k_scan_top(unsigned *__restrict__ bsum, int nb) {
  __shared__ unsigned sh[32];
  const int b0 = threadIdx.x * kScanItems;
  unsigned v[kScanItems], acc = 0;
#pragma unroll
  for (int q = 0; q < kScanItems; q++) {
    v[q] = b0 + q < nb ? bsum[b0 + q] : 0u;
    acc += v[q];
  }
  unsigned total;
  unsigned off = block_excl_scan(acc, sh, total);
#pragma unroll
  for (int q = 0; q < kScanItems; q++) {
    if (b0 + q < nb) bsum[b0 + q] = off;
    off += v[q];
  }
}

// Adds the block offsets; writes the offsets twice (bucket starts and the
// scatter cursors) and the end offset off[n] = total particles.
__global__ void k_scan_add(unsigned *__restrict__ off, unsigned *__restrict__ cursor, long long n,
                           const unsigned *__restrict__ bsum, unsigned total) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i <= n; i += stride) {
    const unsigned v = i < n ? off[i] + bsum[i / kScanChunk] : total;
    off[i] = v;
    if (i < n) cursor[i] = v;
  }
}

// Particle indices bucketed by tile (order inside a tile: the order in which
// warps claim their slots); with `lat` (a single box), also the lattice
// point of every slot, lat[slot] = q[p] (p when q is NULL), so that the
// deposit and the kick read it in slot order instead of through the index.
__global__ void __launch_bounds__(kThreads) k_tile_scatter(const unsigned *__restrict__ tile_of, long long np,
                                                           unsigned *__restrict__ cursor,
                                                           unsigned *__restrict__ order,
                                                           const unsigned *__restrict__ q,
                                                           unsigned *__restrict__ lat) {
  const int lane = threadIdx.x & 31;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long base = (long long)blockIdx.x * blockDim.x + (threadIdx.x & ~31); base < np; base += stride) {
    const long long p = base + lane;
    const bool on = p < np;
    const unsigned am = __ballot_sync(0xffffffffu, on);
    if (!on) continue;
    const unsigned t = tile_of[p];
    const unsigned same = __match_any_sync(am, t);
    const int leader = __ffs(same) - 1;
    unsigned first = 0;
    if (lane == leader) first = atomicAdd(cursor + t, (unsigned)__popc(same));
    first = __shfl_sync(same, first, leader);
    const unsigned slot = first + __popc(same & ((1u << lane) - 1u));
    order[slot] = (unsigned)p;
    if (lat) lat[slot] = q ? q[p] : (unsigned)p;
  }
}

// PtoMesh (src/auxPM.c:280-357) per tile: the weights of the tile's
// particles (WPAR = (N/Ns)^3 folded into the y factors, auxPM.c:316-317) are
// summed in shared memory over the tile (TX x TX x TZ cells, tile_tx) and
// its +1 halo, [TX+1][TX+1][TZ+2] floats (the z rows padded to an even
// length), and the copy is added to the mesh (pre-set to -1) with one float2
// reduction per pair of cells in z, skipping pairs that received nothing.
// Mesh rows have even length and z0 is a multiple of TZ, so every pair is
// 8-byte aligned; with N a multiple of TZ a pair never straddles the
// periodic wrap.
template <int T, bool P2>
__global__ void __launch_bounds__(kThreads) k_cic_tiles(const float *__restrict__ s, const mgp_dstate *__restrict__ st,
                                                        long long np, int Ns, int ls, int N, float scale, float wpar,
                                                        float *__restrict__ rho, long long P,
                                                        const unsigned *__restrict__ off,
                                                        const unsigned *__restrict__ order,
                                                        const unsigned *__restrict__ qs, int ntx, int ntz, int nbox,
                                                        long long g_bs) {
  constexpr int KX = tile_tx(T), KZ = T, BX = KX + 1, BZ = KZ + 2, BOX = BX * BX * BZ;
  __shared__ float box[BOX];
  const float inv_ns = 1.0f / (float)Ns;
  const int ntiles = ntx * ntx * ntz;
  const float *s0 = s;
  const mgp_dstate *st0 = st;
  float *rho0 = rho;
  for (int L = blockIdx.x; L < ntiles * nbox; L += gridDim.x) {
    // box ib of a batch: particles 3 np apart, grids g_bs floats apart; the
    // order holds global particle indices ib np + p
    const int ib = L / ntiles, tile = tile_at(L - ib * ntiles, ntx, ntz), gtile = ib * ntiles + tile;
    const unsigned j0 = off[gtile], j1 = off[gtile + 1];
    if (j0 == j1) continue;
    s = s0 + (long long)ib * 3 * np;
    st = st0 + ib;
    rho = rho0 + (long long)ib * g_bs;
    const long long pbase = (long long)ib * np;
    const float ox = (float)(st->cx[0] * scale), oy = (float)(st->cx[1] * scale), oz = (float)(st->cx[2] * scale);
    const int tz = tile % ntz, ty = (tile / ntz) % ntx, tx = tile / (ntz * ntx);
    const int x0 = tx * KX, y0 = ty * KX, z0 = tz * KZ;
    for (int e = threadIdx.x; e < BOX; e += blockDim.x) box[e] = 0.0f;
    __syncthreads();
    for (unsigned j = j0 + threadIdx.x; j < j1; j += blockDim.x) {
      const long long p = (long long)order[j] - pbase;  // slot of the j-th particle of the tile order
      int ix, iy, iz;
      float DX, DY, DZ;
      particle_cell<P2>(s, np, p, qs ? qs[j] : (unsigned)p, Ns, ls, inv_ns, N, scale, ox, oy, oz, ix, iy, iz, DX,
                        DY, DZ);
      const float TX = 1.0f - DX, TY = (1.0f - DY) * wpar, TZ = 1.0f - DZ;
      DY *= wpar;
      const int lx = ix - x0, ly = iy - y0, lz = iz - z0;
      if ((unsigned)lx >= (unsigned)KX || (unsigned)ly >= (unsigned)KX || (unsigned)lz >= (unsigned)KZ) {
        // a base cell outside the tile (the key pass rounded differently):
        // straight to the mesh
        const int ixn = ix + 1 == N ? 0 : ix + 1, iyn = iy + 1 == N ? 0 : iy + 1, izn = iz + 1 == N ? 0 : iz + 1;
        float *r00 = rho + ((long long)ix * N + iy) * P, *r01 = rho + ((long long)ix * N + iyn) * P;
        float *r10 = rho + ((long long)ixn * N + iy) * P, *r11 = rho + ((long long)ixn * N + iyn) * P;
        atomicAdd(r00 + iz, TX * TY * TZ);
        atomicAdd(r00 + izn, TX * TY * DZ);
        atomicAdd(r01 + iz, TX * DY * TZ);
        atomicAdd(r01 + izn, TX * DY * DZ);
        atomicAdd(r10 + iz, DX * TY * TZ);
        atomicAdd(r10 + izn, DX * TY * DZ);
        atomicAdd(r11 + iz, DX * DY * TZ);
        atomicAdd(r11 + izn, DX * DY * DZ);
        continue;
      }
      const int b = (lx * BX + ly) * BZ + lz;
      atomicAdd(box + b, TX * TY * TZ);
      atomicAdd(box + b + 1, TX * TY * DZ);
      atomicAdd(box + b + BZ, TX * DY * TZ);
      atomicAdd(box + b + BZ + 1, TX * DY * DZ);
      atomicAdd(box + b + BX * BZ, DX * TY * TZ);
      atomicAdd(box + b + BX * BZ + 1, DX * TY * DZ);
      atomicAdd(box + b + BX * BZ + BZ, DX * DY * TZ);
      atomicAdd(box + b + BX * BZ + BZ + 1, DX * DY * DZ);
    }
    __syncthreads();
    for (int e = threadIdx.x; e < BX * BX * (BZ / 2); e += blockDim.x) {
      const int zz = e % (BZ / 2), r = e / (BZ / 2), yy = r % BX, xx = r / BX;
      const float2 v = make_float2(box[r * BZ + 2 * zz], box[r * BZ + 2 * zz + 1]);
      if (v.x == 0.0f && v.y == 0.0f) continue;
      int gx = x0 + xx, gy = y0 + yy, gz = z0 + 2 * zz;
      if (gx >= N) gx -= N;
      if (gy >= N) gy -= N;
      if (gz >= N) gz -= N;
      atomicAdd(reinterpret_cast<float2 *>(rho + ((long long)gx * N + gy) * P + gz), v);
    }
    __syncthreads();
  }
}

// The single-box deposit writes each tile's interior cells itself: a tile's
// box [KX+1][KX+1][KZ+2] splits into the interior (x, y < KX, z < KZ), which
// no other tile's box covers, and the halo, kept as float2 pairs along z
// (z even): face x = KX (all y, all z), face y = KX (x < KX, all z), and the
// pair (KZ, KZ+1) of the interior rows.  The last column of the box (z =
// KZ+1) only pads the rows to an even length and stays zero.
template <int T>
struct tile_halo {
  static constexpr int KX = tile_tx(T), KZ = T, BX = KX + 1, BZ = KZ + 2, RP = BZ / 2;  // pairs per box row
  static constexpr int FX = BX * RP, FY = KX * RP, FZ = KX * KX, PAIRS = FX + FY + FZ;
};

// Box cell (xx, yy, zz) of halo pair h (zz even).
template <int T>
__device__ __forceinline__ void halo_pair(int h, int &xx, int &yy, int &zz) {
  using H = tile_halo<T>;
  if (h < H::FX) {
    xx = H::KX;
    yy = h / H::RP;
    zz = 2 * (h - yy * H::RP);
  } else if (h < H::FX + H::FY) {
    const int g = h - H::FX;
    xx = g / H::RP;
    yy = H::KX;
    zz = 2 * (g - xx * H::RP);
  } else {
    const int g = h - H::FX - H::FY;
    xx = g / H::KX;
    yy = g - xx * H::KX;
    zz = H::KZ;
  }
}

// PtoMesh (src/auxPM.c:280-357) per tile, owner writes (single box): the
// tile's particles are summed in shared memory as in k_cic_tiles, then the
// block stores its interior cells as box - 1 with plain stores (the mesh
// needs no pre-set; every tile stores its interior, empty or not, and the
// last tile in z also sets the row padding to -1 as a fill would), and writes
// its halo pairs to `halo` (PAIRS per tile).  k_cic_halo then adds the halos
// to the neighbours' interiors.  A particle whose base cell falls outside its
// tile after all (not expected: the key pass rounds identically) is listed in
// `spill` for k_cic_halo, after every interior has been stored.
template <int T, bool P2>
__global__ void __launch_bounds__(kThreads) k_cic_tiles_own(const float *__restrict__ s,
                                                            const mgp_dstate *__restrict__ st, long long np, int Ns,
                                                            int ls, int N, float scale, float wpar,
                                                            float *__restrict__ rho, long long P,
                                                            const unsigned *__restrict__ off,
                                                            const unsigned *__restrict__ order,
                                                            const unsigned *__restrict__ qs, int ntx, int ntz,
                                                            float2 *__restrict__ halo, unsigned *__restrict__ spill,
                                                            unsigned *__restrict__ nspill) {
  using H = tile_halo<T>;
  constexpr int KX = H::KX, KZ = H::KZ, BX = H::BX, BZ = H::BZ, BOX = BX * BX * BZ;
  __shared__ __align__(16) float box[BOX];
  const float inv_ns = 1.0f / (float)Ns;
  const int ntiles = ntx * ntx * ntz;
  const float ox = (float)(st->cx[0] * scale), oy = (float)(st->cx[1] * scale), oz = (float)(st->cx[2] * scale);
  for (int L = blockIdx.x; L < ntiles; L += gridDim.x) {
    const int tile = tile_at(L, ntx, ntz);
    const unsigned j0 = off[tile], j1 = off[tile + 1];
    const int tz = tile % ntz, ty = (tile / ntz) % ntx, tx = tile / (ntz * ntx);
    const int x0 = tx * KX, y0 = ty * KX, z0 = tz * KZ;
    for (int e = threadIdx.x; e < BOX; e += blockDim.x) box[e] = 0.0f;
    __syncthreads();
    for (unsigned j = j0 + threadIdx.x; j < j1; j += blockDim.x) {
      const long long p = (long long)order[j];
      int ix, iy, iz;
      float DX, DY, DZ;
      particle_cell<P2>(s, np, p, qs[j], Ns, ls, inv_ns, N, scale, ox, oy, oz, ix, iy, iz, DX, DY, DZ);
      const float TX = 1.0f - DX, TY = (1.0f - DY) * wpar, TZ = 1.0f - DZ;
      DY *= wpar;
      const int lx = ix - x0, ly = iy - y0, lz = iz - z0;
      if ((unsigned)lx >= (unsigned)KX || (unsigned)ly >= (unsigned)KX || (unsigned)lz >= (unsigned)KZ) {
        spill[atomicAdd(nspill, 1u)] = j;  // at most np entries: every slot once
        continue;
      }
      const int b = (lx * BX + ly) * BZ + lz;
      atomicAdd(box + b, TX * TY * TZ);
      atomicAdd(box + b + 1, TX * TY * DZ);
      atomicAdd(box + b + BZ, TX * DY * TZ);
      atomicAdd(box + b + BZ + 1, TX * DY * DZ);
      atomicAdd(box + b + BX * BZ, DX * TY * TZ);
      atomicAdd(box + b + BX * BZ + 1, DX * TY * DZ);
      atomicAdd(box + b + BX * BZ + BZ, DX * DY * TZ);
      atomicAdd(box + b + BX * BZ + BZ + 1, DX * DY * DZ);
    }
    __syncthreads();
    // interior: rows of the mesh have even length and z0 is even, so every
    // pair is 8-byte aligned
    for (int e = threadIdx.x; e < KX * KX * (KZ / 2); e += blockDim.x) {
      const int zp = e % (KZ / 2), r = e / (KZ / 2), yy = r % KX, xx = r / KX;
      const float2 v = *reinterpret_cast<const float2 *>(box + (xx * BX + yy) * BZ + 2 * zp);
      *reinterpret_cast<float2 *>(rho + ((long long)(x0 + xx) * N + (y0 + yy)) * P + z0 + 2 * zp) =
          make_float2(v.x - 1.0f, v.y - 1.0f);
    }
    if (z0 + KZ == N) {
      for (int r = threadIdx.x; r < KX * KX; r += blockDim.x) {
        const int yy = r % KX, xx = r / KX;
        *reinterpret_cast<float2 *>(rho + ((long long)(x0 + xx) * N + (y0 + yy)) * P + N) = make_float2(-1.0f, -1.0f);
      }
    }
    float2 *hp = halo + (long long)tile * H::PAIRS;
    for (int h = threadIdx.x; h < H::PAIRS; h += blockDim.x) {
      int xx, yy, zz;
      halo_pair<T>(h, xx, yy, zz);
      hp[h] = *reinterpret_cast<const float2 *>(box + (xx * BX + yy) * BZ + zz);
    }
    __syncthreads();  // the box is cleared for the next tile
  }
}

// The halos of k_cic_tiles_own added to the mesh (float2 reductions, zero
// pairs skipped; a pair never straddles the periodic wrap: z0 + KZ is even
// and at most N), then the listed particles straight to the mesh.
template <int T, bool P2>
__global__ void __launch_bounds__(kThreads) k_cic_halo(const float2 *__restrict__ halo, int ntx, int ntz,
                                                       float *__restrict__ rho, long long P,
                                                       const float *__restrict__ s,
                                                       const mgp_dstate *__restrict__ st, long long np, int Ns,
                                                       int ls, int N, float scale, float wpar,
                                                       const unsigned *__restrict__ order,
                                                       const unsigned *__restrict__ qs,
                                                       const unsigned *__restrict__ spill,
                                                       const unsigned *__restrict__ nspill) {
  using H = tile_halo<T>;
  const long long n = (long long)ntx * ntx * ntz * H::PAIRS;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const float2 v = halo[i];
    if (v.x == 0.0f && v.y == 0.0f) continue;
    const int tile = (int)(i / H::PAIRS), h = (int)(i - (long long)tile * H::PAIRS);
    int xx, yy, zz;
    halo_pair<T>(h, xx, yy, zz);
    const int tz = tile % ntz, ty = (tile / ntz) % ntx, tx = tile / (ntz * ntx);
    int gx = tx * H::KX + xx, gy = ty * H::KX + yy, gz = tz * H::KZ + zz;
    if (gx >= N) gx -= N;
    if (gy >= N) gy -= N;
    if (gz >= N) gz -= N;
    atomicAdd(reinterpret_cast<float2 *>(rho + ((long long)gx * N + gy) * P + gz), v);
  }
  const unsigned ns = *nspill;
  if (ns == 0) return;
  const float inv_ns = 1.0f / (float)Ns;
  const float ox = (float)(st->cx[0] * scale), oy = (float)(st->cx[1] * scale), oz = (float)(st->cx[2] * scale);
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < (long long)ns; k += stride) {
    const unsigned j = spill[k];
    int ix, iy, iz;
    float DX, DY, DZ;
    particle_cell<P2>(s, np, (long long)order[j], qs[j], Ns, ls, inv_ns, N, scale, ox, oy, oz, ix, iy, iz, DX, DY,
                      DZ);
    const float TX = 1.0f - DX, TY = (1.0f - DY) * wpar, TZ = 1.0f - DZ;
    DY *= wpar;
    const int ixn = ix + 1 == N ? 0 : ix + 1, iyn = iy + 1 == N ? 0 : iy + 1, izn = iz + 1 == N ? 0 : iz + 1;
    float *r00 = rho + ((long long)ix * N + iy) * P, *r01 = rho + ((long long)ix * N + iyn) * P;
    float *r10 = rho + ((long long)ixn * N + iy) * P, *r11 = rho + ((long long)ixn * N + iyn) * P;
    atomicAdd(r00 + iz, TX * TY * TZ);
    atomicAdd(r00 + izn, TX * TY * DZ);
    atomicAdd(r01 + iz, TX * DY * TZ);
    atomicAdd(r01 + izn, TX * DY * DZ);
    atomicAdd(r10 + iz, DX * TY * TZ);
    atomicAdd(r10 + izn, DX * TY * DZ);
    atomicAdd(r11 + iz, DX * DY * TZ);
    atomicAdd(r11 + izn, DX * DY * DZ);
  }
}

// Back to lattice order: the particle of slot j goes to slot q[j] (D1 and
// D2 are never permuted).
__global__ void __launch_bounds__(kThreads) k_unpermute(long long np, const float *__restrict__ s,
                                                        const float *__restrict__ v, const unsigned *__restrict__ q,
                                                        float *__restrict__ s2, float *__restrict__ v2) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x; j < np; j += stride) {
    const long long dst = q[j];
#pragma unroll
    for (int a = 0; a < 3; a++) {
      const long long o = a * np;
      s2[o + dst] = s[o + j];
      v2[o + dst] = v[o + j];
    }
  }
}

// The LPT displacements of every particle packed in lattice order, 32 bytes
// each: (D1x, D1y, D1z, D2x), (D2y, D2z, 0, 0) -- one sector per particle
// for the tile kick's reads through q.
__global__ void __launch_bounds__(kThreads) k_pack_lpt(long long np, const float *__restrict__ D1,
                                                       const float *__restrict__ D2, float4 *__restrict__ lpt) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < np; p += stride) {
    lpt[2 * p] = make_float4(D1[p], D1[np + p], D1[2 * np + p], D2[p]);
    lpt[2 * p + 1] = make_float4(D2[np + p], D2[2 * np + p], 0.0f, 0.0f);
  }
}

// Block sum of one double per thread (the result in thread 0).
__device__ __forceinline__ double block_sum_tiles(double x, double *sh) {
  for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) sh[w] = x;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x == 0)
    for (int k = 0; k < (int)(blockDim.x >> 5); k++) t += sh[k];
  return t;
}

// Force tile in shared memory: three components, each (TX+1)^2 rows of
// R = TZ + 4 floats (tile shape TX x TX x TZ, tile_tx).  A grid row (x, y)
// of N + 2 floats starts on a 16-byte boundary when y is even and 8 bytes
// past one when y is odd, so row (xx, yy) of the tile is copied as R/4
// 16-byte pieces from z0 (yy even) or z0 - 2 (yy odd): the tile's
// z0..z0+TZ then sit at offset 2 (yy & 1) of the row.  The copied run stays inside the grids: an odd row's starts 2 floats
// into the previous row's padding, an even row's ends at most 2 floats into
// the next row (y <= N - 2).  The z halo of the last tile in z lands in the
// row padding and is patched from z = 0.
template <int T>
struct force_tile {
  static constexpr int TX = tile_tx(T), TZ = T;
  static constexpr int X = TX + 1, R = TZ + 4, COMP = X * X * R, FLOATS = 3 * COMP;
  static constexpr int PIECES = R / 4;  // 16-byte copies per row
};

// Shared-memory offset of row (xx, yy) of component c of the force tile
// (the element z0 + zz is at the returned offset + zz).
template <int T>
__device__ __forceinline__ int tile_row(int c, int xx, int yy) {
  using FT = force_tile<T>;
  return c * FT::COMP + (xx * FT::X + yy) * FT::R + 2 * (yy & 1);
}

// MtoParticles (src/auxPM.c:560-644) + Kick (src/main.c:688-742) + Drift
// (src/main.c:747-787) per cell tile, writing the particles in tile order.
// Tile `tile` holds order[off[tile] .. off[tile+1]), the slots of the
// particles whose CIC base cell lies in it (k_tile_key, same positions).
// The block copies fx, fy, fz over the tile's cells and the +1 halo
// (periodic) into shared memory (force_tile), then for each particle:
// reads slot p = order[j] of the input arrays and its lattice point qs[j]
// (written by the sort's scatter), interpolates the forces from
// shared memory (a base cell outside the tile -- not expected, the key pass
// rounds identically -- reads the global grids), kicks and drifts as
// k_interp_kick_drift does (same expressions in the same order), and writes
// slot j of the output arrays (s, v; qs is the new order's lattice map).  D1/D2
// (scale-independent growth) stay in lattice order, packed 32 bytes per
// particle in `lpt` and read through the lattice point.  Per-block sums of the
// interpolated forces and new velocities go to partials for k_finalize_kd.
// PI: particle-array offset type, 32-bit when 3 np < 2^32 (fewer integer
// instructions per access); NT: threads per block (512: two blocks per SM
// within 64 registers a thread).
template <int T, bool P2, typename PI, int NT>
__global__ void __launch_bounds__(NT, NT >= 512 ? 2 : 0) k_ikd_tiles(
    const float *__restrict__ frc, long long gf, int N, long long P, int Ns, int ls, long long np,
    const float *__restrict__ s, const float *__restrict__ v, const float4 *__restrict__ lpt,
    const unsigned *__restrict__ qs, const unsigned *__restrict__ off, const unsigned *__restrict__ order, int ntx,
    int ntz, const mgp_dstate *__restrict__ st, float *__restrict__ s2, float *__restrict__ v2,
    double *__restrict__ partials, mgp_kd_args a) {
  using FT = force_tile<T>;
  constexpr int X = FT::X, R = FT::R, COMP = FT::COMP, K = FT::PIECES, KX = FT::TX, KZ = FT::TZ;
  constexpr int ROWS = NT / K;  // rows copied per pass of the block
  extern __shared__ __align__(16) float fs[];  // FT::FLOATS
  __shared__ double sh[NT / 32];
  __shared__ long long rowoff[X * X];  // grid offset of row (x0 + xx, y0 + yy), periodic
  const int sub = threadIdx.x / K, k = threadIdx.x - sub * K;  // this thread's row in a pass, its piece
  const float ox = (float)(st->cx[0] * a.scale), oy = (float)(st->cx[1] * a.scale), oz = (float)(st->cx[2] * a.scale);
  const float inv_ns = 1.0f / (float)Ns;
  const int ntiles = ntx * ntx * ntz;
  float accD[3] = {0.f, 0.f, 0.f}, accV[3] = {0.f, 0.f, 0.f};
  for (int L = blockIdx.x; L < ntiles; L += gridDim.x) {
    const int tile = tile_at(L, ntx, ntz);
    const unsigned j0 = off[tile], j1 = off[tile + 1];
    if (j0 == j1) continue;
    const int tz = tile % ntz, ty = (tile / ntz) % ntx, tx = tile / (ntz * ntx);
    const int x0 = tx * KX, y0 = ty * KX, z0 = tz * KZ;
    __syncthreads();  // the previous tile's reads of fs and rowoff are done
    for (int r = threadIdx.x; r < X * X; r += NT) {
      const int xx = r / X, yy = r - xx * X;
      const int gx = x0 + xx >= N ? x0 + xx - N : x0 + xx, gy = y0 + yy >= N ? y0 + yy - N : y0 + yy;
      rowoff[r] = ((long long)gx * N + gy) * P + z0 - 2 * (yy & 1);
    }
    __syncthreads();
    if (sub < ROWS) {
      for (int r = sub; r < 3 * X * X; r += ROWS) {
        const int c = r >= 2 * X * X ? 2 : (r >= X * X ? 1 : 0), rr = r - c * X * X;
        cp_async16(fs + c * COMP + rr * R + 4 * k, frc + c * gf + rowoff[rr] + 4 * k);
      }
    }
    cp_async_wait_all();
    __syncthreads();
    if (z0 + KZ == N) {
      // last tile in z: the halo column z0 + KZ is z = 0 of the same row
      for (int r = threadIdx.x; r < 3 * X * X; r += NT) {
        const int c = r / (X * X), rr = r - c * X * X, yy = rr % X;
        fs[c * COMP + rr * R + 2 * (yy & 1) + KZ] = frc[c * gf + rowoff[rr] + 2 * (yy & 1) - z0];
      }
      __syncthreads();
    }
    const PI npi = (PI)np;
    for (unsigned j = j0 + threadIdx.x; j < j1; j += blockDim.x) {
      const PI p = (PI)order[j];
      const unsigned lat = qs[j];
      const float sp[3] = {s[p], s[npi + p], s[2 * npi + p]};
      const float4 l0 = lpt[2 * (size_t)lat], l1 = lpt[2 * (size_t)lat + 1];
      const float D1p[3] = {l0.x, l0.y, l0.z}, D2p[3] = {l0.w, l1.x, l1.y};
      int ix, iy, iz;
      float DX, DY, DZ;
      cell_of<P2>(sp[0], sp[1], sp[2], lat, Ns, ls, inv_ns, N, a.scale, ox, oy, oz, ix, iy, iz, DX, DY, DZ);
      const float TX = 1.0f - DX, TY = 1.0f - DY, TZ = 1.0f - DZ;
      const float w000 = TX * TY * TZ, w001 = TX * TY * DZ, w010 = TX * DY * TZ, w011 = TX * DY * DZ;
      const float w100 = DX * TY * TZ, w101 = DX * TY * DZ, w110 = DX * DY * TZ, w111 = DX * DY * DZ;
      const int lx = ix - x0, ly = iy - y0, lz = iz - z0;
      float disp[3];
      if ((unsigned)lx < (unsigned)KX && (unsigned)ly < (unsigned)KX && (unsigned)lz < (unsigned)KZ) {
        // row (lx, ly + 1) is in the other parity's box
        const float *f = fs + tile_row<T>(0, lx, ly) + lz;
        const int dy = R + ((ly & 1) ? -2 : 2), dx = X * R;
#pragma unroll
        for (int c = 0; c < 3; c++) {
          const float *F = f + c * COMP;
          disp[c] = F[0] * w000 + F[1] * w001 + F[dy] * w010 + F[dy + 1] * w011 + F[dx] * w100 + F[dx + 1] * w101 +
                    F[dx + dy] * w110 + F[dx + dy + 1] * w111;
        }
      } else {
        const long long xa = (long long)ix * N * P, xb = (ix + 1 == N ? 0 : (long long)(ix + 1) * N * P);
        const long long ya = (long long)iy * P, yb = (iy + 1 == N ? 0 : (long long)(iy + 1) * P);
        const long long za = iz, zb = iz + 1 == N ? 0 : iz + 1;
#pragma unroll
        for (int c = 0; c < 3; c++) {
          const float *F = frc + c * gf;
          disp[c] = F[xa + ya + za] * w000 + F[xa + ya + zb] * w001 + F[xa + yb + za] * w010 +
                    F[xa + yb + zb] * w011 + F[xb + ya + za] * w100 + F[xb + ya + zb] * w101 +
                    F[xb + yb + za] * w110 + F[xb + yb + zb] * w111;
        }
      }
#pragma unroll
      for (int ax = 0; ax < 3; ax++) {
        const PI o = (PI)ax * npi, oj = o + (PI)j;
        const float d1 = D1p[ax], d2 = D2p[ax];
        const float vn = v[o + p] + a.kick_disp * disp[ax] + a.kick_d1 * d1 + a.kick_d2 * d2;
        v2[oj] = vn;
        s2[oj] = a.do_drift ? sp[ax] + vn * a.dyyy + a.dD1 * d1 + a.dD2 * d2 : sp[ax];
        accD[ax] += disp[ax];
        accV[ax] += vn;
      }
    }
  }
#pragma unroll
  for (int c = 0; c < 3; c++) {
    double t = block_sum_tiles((double)accD[c], sh);
    if (threadIdx.x == 0) partials[(long long)blockIdx.x * 6 + c] = t;
    t = block_sum_tiles((double)accV[c], sh);
    if (threadIdx.x == 0) partials[(long long)blockIdx.x * 6 + 3 + c] = t;
  }
}

}  // namespace

// Tile shape of the single-box tile path, or 0 when it does not apply (the
// mesh must split into whole tiles and the indices fit 32 bits): 8 x 8 x 64
// cells (kElong) for meshes of 512 and more (rows of 256 bytes in the
// deposit's flush and the kick's staging), else 16^3 or 8^3.
int mgp_tile_side(int N, long long np) {
  if (np <= 0 || np > 0xffffffffLL) return 0;
  if (N >= 512 && N % kElong == 0) return kElong;
  if (N >= 64 && N % 16 == 0) return 16;
  if (N >= 16 && N % 8 == 0) return 8;
  return 0;
}

// Whether the tile deposit of shape T (8 or 16: T^3 cells; kElong: 8 x 8 x
// 64) applies to the context's boxes: whole tiles, particle indices of all
// boxes in 32 bits, the tiles of all boxes within the two-level scan
// (kScanChunk^2).
int mgp_tiles_check(const mgp_ctx *c, int T) {
  if (T != 8 && T != 16 && T != kElong) return mgp_set_error(MGP_EINVAL, "tile shape %d (8, 16 or %d)", T, kElong);
  if (c->g.N % T) return mgp_set_error(MGP_EINVAL, "tile shape %d does not divide Nmesh = %d", T, c->g.N);
  const long long ntx = c->g.N / tile_tx(T), ntz = c->g.N / T;
  const long long ntiles = ntx * ntx * ntz * c->nbox, nall = c->np * c->nbox;
  if (nall > 0xffffffffLL) return mgp_set_error(MGP_EINVAL, "%lld particles exceed 32-bit indices", nall);
  if (ntiles > (long long)kScanChunk * kScanChunk)
    return mgp_set_error(MGP_EINVAL, "%lld tiles exceed the scan's capacity", ntiles);
  return MGP_OK;
}

// Tile arrays for side T over all boxes of the context (the count and
// offset arrays grow when a batch tries a smaller tile side).
int mgp_tiles_alloc(mgp_ctx *c, int T) {
  int rc = mgp_tiles_check(c, T);
  if (rc != MGP_OK) return rc;
  const int nt1 = c->g.N / tile_tx(T), ntz = c->g.N / T;
  const long long ntiles = (long long)nt1 * nt1 * ntz * c->nbox, nall = c->np * c->nbox;
  const long long nblk = (ntiles + kScanChunk - 1) / kScanChunk;
  if (!c->tile_order) {
    MGP_CUDA(cudaMalloc(&c->tile_of, sizeof(unsigned) * (size_t)nall));
    MGP_CUDA(cudaMalloc(&c->tile_order, sizeof(unsigned) * (size_t)nall));
  }
  if (c->nbox == 1 && !c->q) {
    // q: lattice point of every slot of the particle arrays (in tile order
    // after a tile kick); q_alt: the same for the slots of the last sort
    MGP_CUDA(cudaMalloc(&c->q, sizeof(unsigned) * (size_t)c->np));
    MGP_CUDA(cudaMalloc(&c->q_alt, sizeof(unsigned) * (size_t)c->np));
  }
  if (ntiles > c->tile_cap) {
    void *b[] = {c->tile_count, c->tile_off, c->tile_cursor, c->tile_bsum};
    for (void *x : b)
      if (x) cudaFree(x);
    MGP_CUDA(cudaMalloc(&c->tile_count, sizeof(unsigned) * (size_t)ntiles));
    MGP_CUDA(cudaMalloc(&c->tile_off, sizeof(unsigned) * (size_t)(ntiles + 1)));
    MGP_CUDA(cudaMalloc(&c->tile_cursor, sizeof(unsigned) * (size_t)ntiles));
    MGP_CUDA(cudaMalloc(&c->tile_bsum, sizeof(unsigned) * (size_t)nblk));
    c->tile_cap = ntiles;
  }
  c->tile_side = T;
  c->tile_n1 = nt1;
  c->tile_nz = ntz;
  return MGP_OK;
}

void mgp_tiles_free(mgp_ctx *c) {
  void *b[] = {c->tile_of, c->tile_order, c->tile_count, c->tile_off, c->tile_cursor, c->tile_bsum,
               c->q, c->q_alt, c->s_alt, c->v_alt, c->lpt, c->tile_halo, c->tile_spill};
  for (void *x : b)
    if (x) cudaFree(x);
  c->tile_halo = NULL;
  c->tile_spill = NULL;
  c->tile_halo_bytes = 0;
  c->tile_of = c->tile_order = c->tile_count = c->tile_off = c->tile_cursor = c->tile_bsum = NULL;
  c->q = c->q_alt = NULL;
  c->s_alt = c->v_alt = c->lpt = NULL;
  c->lpt_built = -1;
  c->tile_ready = 0;
  c->tile_cap = 0;
  c->permuted = 0;
}

static void swap_arrays(mgp_ctx *c) {
  float *t;
  t = c->s; c->s = c->s_alt; c->s_alt = t;
  t = c->v; c->v = c->v_alt; c->v_alt = t;
}

// Lattice order of the particle arrays (the particle of slot j to slot
// q[j]); every caller of this is about to read or replace the particles, so
// the last tile sort no longer describes the arrays.
int mgp_particles_canonical(mgp_ctx *c) {
  c->tile_ready = 0;
  if (!c->permuted) return MGP_OK;
  k_unpermute<<<mgp_blocks_for(c->np, 8), kThreads, 0, c->stream>>>(c->np, c->s, c->v, c->q, c->s_alt, c->v_alt);
  MGP_CHECK_LAUNCH();
  g_kernel_launches++;
  swap_arrays(c);
  c->permuted = 0;
  return MGP_OK;
}

// Bucket the particles of every box by tile of side T (their current
// positions).
int mgp_tiles_sort(mgp_ctx *c, int T) {
  int rc = mgp_tiles_alloc(c, T);
  if (rc != MGP_OK) return rc;
  const int N = c->g.N, Ns = c->Ns, nt1 = c->tile_n1, ntz = c->tile_nz, B = c->nbox;
  const long long ntiles = (long long)nt1 * nt1 * ntz * B, nall = c->np * B;
  const int ls = lattice_log2(Ns);
  const float scale = (float)(N / c->p.Box);
  int sx = 0, sz = 0;
  while ((1 << sx) < tile_tx(T)) sx++;
  while ((1 << sz) < T) sz++;
  const unsigned *qp = c->permuted ? c->q : NULL;
  MGP_CUDA(cudaMemsetAsync(c->tile_count, 0, sizeof(unsigned) * (size_t)ntiles, c->stream));
  const dim3 gk(mgp_blocks_per_box(c->np, 8, B), B);
  if (ls >= 0)
    k_tile_key<true><<<gk, kThreads, 0, c->stream>>>(c->s, c->dstate, c->np, Ns, ls, N, scale, sx, sz, nt1, ntz, qp,
                                                     c->tile_of, c->tile_count);
  else
    k_tile_key<false><<<gk, kThreads, 0, c->stream>>>(c->s, c->dstate, c->np, Ns, ls, N, scale, sx, sz, nt1, ntz, qp,
                                                      c->tile_of, c->tile_count);
  MGP_CHECK_LAUNCH();
  g_kernel_launches++;
  const int nblk = (int)((ntiles + kScanChunk - 1) / kScanChunk);
  k_scan_local<<<nblk, kThreads, 0, c->stream>>>(c->tile_count, ntiles, c->tile_off, c->tile_bsum);
  MGP_CHECK_LAUNCH();
  g_kernel_launches++;
  k_scan_top<<<1, kThreads, 0, c->stream>>>(c->tile_bsum, nblk);
  MGP_CHECK_LAUNCH();
  g_kernel_launches++;
  k_scan_add<<<mgp_blocks_for(ntiles + 1, 8), kThreads, 0, c->stream>>>(c->tile_off, c->tile_cursor, ntiles,
                                                                        c->tile_bsum, (unsigned)nall);
  MGP_CHECK_LAUNCH();
  g_kernel_launches++;
  k_tile_scatter<<<mgp_blocks_for(nall, 8), kThreads, 0, c->stream>>>(
      c->tile_of, nall, c->tile_cursor, c->tile_order, qp, c->nbox == 1 ? c->q_alt : NULL);
  MGP_CHECK_LAUNCH();
  g_kernel_launches++;
  c->tile_ready = 1;
  return MGP_OK;
}

// Tile deposit onto meshes pre-set to -1 (after mgp_tiles_sort); per_sm:
// resident blocks per SM of the launch (0: the default budget).
int mgp_cic_tiles(mgp_ctx *c, float wpar, int per_sm) {
  // lattice point of every slot of the sort (single box), else the slot's own
  const unsigned *ord = c->tile_order, *qs = c->nbox == 1 ? c->q_alt : NULL;
  const int N = c->g.N, Ns = c->Ns, T = c->tile_side, nt1 = c->tile_n1, ntz = c->tile_nz, B = c->nbox;
  const long long gbs = c->g.nreal;
  const int ls = lattice_log2(Ns);
  const float scale = (float)(N / c->p.Box);
  const int nb = mgp_blocks_for((long long)nt1 * nt1 * ntz * B * kThreads, per_sm > 0 ? per_sm : 8);
#define MGP_CIC_TILES(TT, PP)                                                                                 \
  k_cic_tiles<TT, PP><<<nb, kThreads, 0, c->stream>>>(c->s, c->dstate, c->np, Ns, ls, N, scale, wpar, c->rho, \
                                                      c->g.P, c->tile_off, ord, qs, nt1, ntz, B, gbs)
  if (T == kElong && ls >= 0)
    MGP_CIC_TILES(kElong, true);
  else if (T == kElong)
    MGP_CIC_TILES(kElong, false);
  else if (T == 16 && ls >= 0)
    MGP_CIC_TILES(16, true);
  else if (T == 16)
    MGP_CIC_TILES(16, false);
  else if (ls >= 0)
    MGP_CIC_TILES(8, true);
  else
    MGP_CIC_TILES(8, false);
#undef MGP_CIC_TILES
  MGP_CHECK_LAUNCH();
  g_kernel_launches++;
  return MGP_OK;
}

// Single-box tile deposit with owner writes (after mgp_tiles_sort; the
// mesh needs no pre-set): k_cic_tiles_own stores every tile's interior and
// its halo pairs, k_cic_halo adds the halos and the listed particles.
int mgp_cic_tiles_own(mgp_ctx *c, float wpar) {
  if (c->nbox != 1 || !c->tile_ready) return mgp_set_error(MGP_ESTATE, "owner-writes deposit without a current tile sort");
  const int N = c->g.N, Ns = c->Ns, T = c->tile_side, nt1 = c->tile_n1, ntz = c->tile_nz;
  if (c->g.P != N + 2) return mgp_set_error(MGP_EINVAL, "mesh rows of %lld floats, expected %d", c->g.P, N + 2);
  const long long ntiles = (long long)nt1 * nt1 * ntz;
  const int pairs = T == kElong ? tile_halo<kElong>::PAIRS : (T == 16 ? tile_halo<16>::PAIRS : tile_halo<8>::PAIRS);
  const size_t hbytes = sizeof(float2) * (size_t)ntiles * (size_t)pairs;
  if (hbytes > c->tile_halo_bytes) {
    if (c->tile_halo) cudaFree(c->tile_halo);
    c->tile_halo = NULL;
    c->tile_halo_bytes = 0;
    MGP_CUDA(cudaMalloc(&c->tile_halo, hbytes));
    c->tile_halo_bytes = hbytes;
  }
  if (!c->tile_spill) {
    MGP_CUDA(cudaMalloc(&c->tile_spill, sizeof(unsigned) * ((size_t)c->np + 1)));
  }
  unsigned *nspill = c->tile_spill + c->np;
  MGP_CUDA(cudaMemsetAsync(nspill, 0, sizeof(unsigned), c->stream));
  const int ls = lattice_log2(Ns);
  const float scale = (float)(N / c->p.Box);
  float2 *halo = (float2 *)c->tile_halo;
  const int nb = mgp_blocks_for(ntiles * kThreads, 8);
  const int nh = mgp_blocks_for(ntiles * pairs, 8);
#define MGP_CIC_OWN(TT, PP)                                                                                          \
  do {                                                                                                               \
    k_cic_tiles_own<TT, PP><<<nb, kThreads, 0, c->stream>>>(c->s, c->dstate, c->np, Ns, ls, N, scale, wpar, c->rho, \
                                                            c->g.P, c->tile_off, c->tile_order, c->q_alt, nt1, ntz, \
                                                            halo, c->tile_spill, nspill);                            \
    MGP_CHECK_LAUNCH();                                                                                              \
    g_kernel_launches++;                                                                                             \
    k_cic_halo<TT, PP><<<nh, kThreads, 0, c->stream>>>(halo, nt1, ntz, c->rho, c->g.P, c->s, c->dstate, c->np, Ns,  \
                                                       ls, N, scale, wpar, c->tile_order, c->q_alt, c->tile_spill,   \
                                                       nspill);                                                      \
    MGP_CHECK_LAUNCH();                                                                                              \
    g_kernel_launches++;                                                                                             \
  } while (0)
  if (T == kElong && ls >= 0)
    MGP_CIC_OWN(kElong, true);
  else if (T == kElong)
    MGP_CIC_OWN(kElong, false);
  else if (T == 16 && ls >= 0)
    MGP_CIC_OWN(16, true);
  else if (T == 16)
    MGP_CIC_OWN(16, false);
  else if (ls >= 0)
    MGP_CIC_OWN(8, true);
  else
    MGP_CIC_OWN(8, false);
#undef MGP_CIC_OWN
  return MGP_OK;
}

// Kick + drift per tile in the order of the last mgp_tiles_sort (a single
// box with particle-array LPT displacements; the positions unchanged since
// the sort), the particle arrays rewritten in that order into the second
// buffers, which then become the arrays.  nblocks_out: the grid, whose
// per-block partial sums k_finalize_kd reduces.
int mgp_ikd_tiles(mgp_ctx *c, const mgp_kd_args *a, int *nblocks_out) {
  if (!c->tile_ready || c->nbox != 1) return mgp_set_error(MGP_ESTATE, "tile kick without a current tile sort");
  const size_t bytes = sizeof(float) * 3 * (size_t)c->np;
  if (!c->s_alt) {
    MGP_CUDA(cudaMalloc(&c->s_alt, bytes));
    MGP_CUDA(cudaMalloc(&c->v_alt, bytes));
    MGP_CUDA(cudaMalloc(&c->lpt, sizeof(float) * 8 * (size_t)c->np));
    c->lpt_built = -1;
  }
  if (c->lpt_built != c->lpt_ver) {
    // D1/D2 changed since the last pack (IC, or set by the caller)
    k_pack_lpt<<<mgp_blocks_for(c->np, 8), kThreads, 0, c->stream>>>(c->np, c->D1, c->D2, (float4 *)c->lpt);
    MGP_CHECK_LAUNCH();
    g_kernel_launches++;
    c->lpt_built = c->lpt_ver;
  }
  const int T = c->tile_side, nt1 = c->tile_n1, ntz = c->tile_nz, N = c->g.N, Ns = c->Ns;
  const int ls = lattice_log2(Ns);
  const long long ntiles = (long long)nt1 * nt1 * ntz;
  // forces per block: 16^3 tiles 68 KB (three blocks of 256 threads per
  // SM), 8 x 8 x 64 tiles 65 KB (two blocks of 512), 8^3 tiles 12 KB (eight
  // of 256)
  const size_t smem = sizeof(float) * (T == kElong ? force_tile<kElong>::FLOATS
                                                   : (T == 16 ? force_tile<16>::FLOATS : force_tile<8>::FLOATS));
  int nb = T == kElong ? mgp_blocks_for(ntiles * 256, 2) : mgp_blocks_for(ntiles * 256, T == 8 ? 8 : 3);
  if (nb > c->max_blocks) nb = c->max_blocks;
#define MGP_IKD_TILES(TT, PP, PI)                                                                             \
  do {                                                                                                        \
    constexpr int NTT = TT == kElong ? 512 : 256;                                                             \
    MGP_CUDA(cudaFuncSetAttribute(k_ikd_tiles<TT, PP, PI, NTT>, cudaFuncAttributeMaxDynamicSharedMemorySize,  \
                                  (int)smem));                                                                \
    k_ikd_tiles<TT, PP, PI, NTT><<<nb, NTT, smem, c->stream>>>(c->frc, c->g.nreal, N, c->g.P, Ns, ls, c->np,  \
                                                               c->s, c->v, (const float4 *)c->lpt, c->q_alt,  \
                                                               c->tile_off, c->tile_order, nt1, ntz,          \
                                                               c->dstate, c->s_alt, c->v_alt, c->partials,    \
                                                               *a);                                           \
  } while (0)
  const bool narrow = 3 * c->np < 0xffffffffLL;
  if (T == kElong && ls >= 0 && narrow)
    MGP_IKD_TILES(kElong, true, unsigned);
  else if (T == kElong && ls >= 0)
    MGP_IKD_TILES(kElong, true, long long);
  else if (T == kElong)
    MGP_IKD_TILES(kElong, false, long long);
  else if (T == 16 && ls >= 0 && narrow)
    MGP_IKD_TILES(16, true, unsigned);
  else if (T == 16 && ls >= 0)
    MGP_IKD_TILES(16, true, long long);
  else if (T == 16)
    MGP_IKD_TILES(16, false, long long);
  else if (ls >= 0)
    MGP_IKD_TILES(8, true, long long);
  else
    MGP_IKD_TILES(8, false, long long);
#undef MGP_IKD_TILES
  MGP_CHECK_LAUNCH();
  g_kernel_launches++;
  swap_arrays(c);
  unsigned *t = c->q;
  c->q = c->q_alt;
  c->q_alt = t;
  c->permuted = 1;
  c->tile_ready = 0;  // the arrays are in the sort's order now, the positions drifted
  *nblocks_out = nb;
  return MGP_OK;
}
