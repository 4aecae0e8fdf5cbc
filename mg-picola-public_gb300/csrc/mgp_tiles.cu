// Cell-tile order of the particles for the two particle passes of the PM
// step (sm_103a).
//
// The particle arrays stay in Lagrangian (lattice) order.  Once per step,
// before the deposit, the particles are counted and bucketed by the T^3-cell
// tile of their CIC base cell (a counting sort of the particle indices, 8
// bytes per particle of traffic besides one read of the displacements):
//   k_tile_key      tile of every particle, tile counts (warp-aggregated)
//   k_scan_*        exclusive prefix sum of the counts = tile offsets
//   k_tile_scatter  particle indices bucketed by tile
// Then
//   k_cic_tiles     PtoMesh (src/auxPM.c:280-357): one block per tile
//                   accumulates its particles' CIC weights in a shared-memory
//                   copy of the tile plus its +1 halo, then adds the copy to
//                   the mesh with one vector reduction per pair of cells
//                   (about 1.7 L2 reduction sectors per particle instead of
//                   ~4.3 for eight scalar reductions per particle);
// Any order gives the same density (up to the order of floating-point
// sums); the tile order restores the locality of the deposit that the
// Lagrangian order loses as the particles cluster.
#include <cuda_runtime.h>
#include <stdint.h>

#include "mgp_device.cuh"
#include "mgp_internal.h"

namespace {

constexpr int kThreads = 256;
constexpr int kScanItems = 16;                     // per thread in a scan block
constexpr int kScanChunk = kThreads * kScanItems;  // elements per scan block

// CIC base cell of particle p (the same arithmetic as k_cic), and its tile.
// p is the array slot, lat the lattice point of the particle in it.
template <bool P2>
__device__ __forceinline__ void particle_cell(const float *__restrict__ s, long long np, long long p, unsigned lat,
                                              int Ns, int ls, float inv_ns, int N, float scale, float ox, float oy,
                                              float oz, int &ix, int &iy, int &iz, float &DX, float &DY, float &DZ) {
  int i, j, k;
  if (P2) {
    lattice_ijk_p2(lat, ls, i, j, k);
    cell_frac_p2(i, s[p], ox, N, ls, inv_ns, scale, ix, DX);
    cell_frac_p2(j, s[np + p], oy, N, ls, inv_ns, scale, iy, DY);
    cell_frac_p2(k, s[2 * np + p], oz, N, ls, inv_ns, scale, iz, DZ);
  } else {
    lattice_ijk(lat, Ns, i, j, k);
    cell_frac(i, s[p], ox, N, Ns, scale, ix, DX);
    cell_frac(j, s[np + p], oy, N, Ns, scale, iy, DY);
    cell_frac(k, s[2 * np + p], oz, N, Ns, scale, iz, DZ);
  }
}

// Tile of every particle and the per-tile counts.  The loop runs in whole
// warps (warp-aligned starts, stride a multiple of 32) so that the lanes of
// a warp can merge their count increments per tile.
template <bool P2>
__global__ void __launch_bounds__(kThreads) k_tile_key(const float *__restrict__ s, const mgp_dstate *__restrict__ st,
                                                       long long np, int Ns, int ls, int N, float scale, int tshift,
                                                       int ntile1, const unsigned *__restrict__ q,
                                                       unsigned *__restrict__ tile_of,
                                                       unsigned *__restrict__ count) {
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
    const unsigned t = ((unsigned)(ix >> tshift) * (unsigned)ntile1 + (unsigned)(iy >> tshift)) * (unsigned)ntile1 +
                       (unsigned)(iz >> tshift);
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
// warps claim their slots).
__global__ void __launch_bounds__(kThreads) k_tile_scatter(const unsigned *__restrict__ tile_of, long long np,
                                                           unsigned *__restrict__ cursor,
                                                           unsigned *__restrict__ order) {
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
    order[first + __popc(same & ((1u << lane) - 1u))] = (unsigned)p;
  }
}

// PtoMesh (src/auxPM.c:280-357) per tile: the weights of the tile's
// particles (WPAR = (N/Ns)^3 folded into the y factors, auxPM.c:316-317) are
// summed in shared memory over the tile and its +1 halo, [T+1][T+1][T+2]
// floats (the z rows padded to an even length), and the copy is added to the
// mesh (pre-set to -1) with one float2 reduction per pair of cells in z,
// skipping pairs that received nothing.  Mesh rows have even length and z0
// is a multiple of T, so every pair is 8-byte aligned; with N a multiple of
// T a pair never straddles the periodic wrap.
template <int T, bool P2>
__global__ void __launch_bounds__(kThreads) k_cic_tiles(const float *__restrict__ s, const mgp_dstate *__restrict__ st,
                                                        long long np, int Ns, int ls, int N, float scale, float wpar,
                                                        float *__restrict__ rho, long long P,
                                                        const unsigned *__restrict__ off,
                                                        const unsigned *__restrict__ order,
                                                        const unsigned *__restrict__ q, int ntile1) {
  constexpr int BX = T + 1, BZ = T + 2, BOX = BX * BX * BZ;
  __shared__ float box[BOX];
  const float ox = (float)(st->cx[0] * scale), oy = (float)(st->cx[1] * scale), oz = (float)(st->cx[2] * scale);
  const float inv_ns = 1.0f / (float)Ns;
  const int ntiles = ntile1 * ntile1 * ntile1;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const unsigned j0 = off[tile], j1 = off[tile + 1];
    if (j0 == j1) continue;
    const int tz = tile % ntile1, ty = (tile / ntile1) % ntile1, tx = tile / (ntile1 * ntile1);
    const int x0 = tx * T, y0 = ty * T, z0 = tz * T;
    for (int q = threadIdx.x; q < BOX; q += blockDim.x) box[q] = 0.0f;
    __syncthreads();
    for (unsigned j = j0 + threadIdx.x; j < j1; j += blockDim.x) {
      // slot of the j-th particle of the tile order: order[j], or j itself
      // once the arrays have been permuted into that order
      const long long p = order ? (long long)order[j] : (long long)j;
      int ix, iy, iz;
      float DX, DY, DZ;
      particle_cell<P2>(s, np, p, q ? q[p] : (unsigned)p, Ns, ls, inv_ns, N, scale, ox, oy, oz, ix, iy, iz, DX, DY,
                        DZ);
      const float TX = 1.0f - DX, TY = (1.0f - DY) * wpar, TZ = 1.0f - DZ;
      DY *= wpar;
      const int lx = ix - x0, ly = iy - y0, lz = iz - z0;
      if ((unsigned)lx >= (unsigned)T || (unsigned)ly >= (unsigned)T || (unsigned)lz >= (unsigned)T) {
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
    for (int q = threadIdx.x; q < BX * BX * (BZ / 2); q += blockDim.x) {
      const int zz = q % (BZ / 2), r = q / (BZ / 2), yy = r % BX, xx = r / BX;
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

// Gather of the particle arrays into the tile order: slot j takes the
// particle of slot order[j] (s, v, D1, D2: [3][np] each) and its lattice
// point.  Reads come in runs of lattice neighbours, writes are coalesced.
__global__ void __launch_bounds__(kThreads) k_permute(const unsigned *__restrict__ order, long long np,
                                                      const float *__restrict__ s, const float *__restrict__ v,
                                                      const float *__restrict__ D1, const float *__restrict__ D2,
                                                      const unsigned *__restrict__ q, float *__restrict__ s2,
                                                      float *__restrict__ v2, float *__restrict__ D12,
                                                      float *__restrict__ D22, unsigned *__restrict__ q2) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x; j < np; j += stride) {
    const long long src = order[j];
#pragma unroll
    for (int a = 0; a < 3; a++) {
      const long long o = a * np;
      s2[o + j] = s[o + src];
      v2[o + j] = v[o + src];
      D12[o + j] = D1[o + src];
      D22[o + j] = D2[o + src];
    }
    q2[j] = q ? q[src] : (unsigned)src;
  }
}

// Back to lattice order: the particle of slot j goes to slot q[j].
__global__ void __launch_bounds__(kThreads) k_unpermute(long long np, const float *__restrict__ s,
                                                        const float *__restrict__ v, const float *__restrict__ D1,
                                                        const float *__restrict__ D2, const unsigned *__restrict__ q,
                                                        float *__restrict__ s2, float *__restrict__ v2,
                                                        float *__restrict__ D12, float *__restrict__ D22) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x; j < np; j += stride) {
    const long long dst = q[j];
#pragma unroll
    for (int a = 0; a < 3; a++) {
      const long long o = a * np;
      s2[o + dst] = s[o + j];
      v2[o + dst] = v[o + j];
      D12[o + dst] = D1[o + j];
      D22[o + dst] = D2[o + j];
    }
  }
}

}  // namespace

// Tile side in cells for the tile path, or 0 when it does not apply (the
// mesh must split into whole tiles and the indices fit 32 bits).
int mgp_tile_side(int N, long long np) {
  if (np <= 0 || np > 0xffffffffLL) return 0;
  if (N >= 64 && N % 16 == 0) return 16;
  if (N >= 16 && N % 8 == 0) return 8;
  return 0;
}

int mgp_tiles_alloc(mgp_ctx *c) {
  if (c->tile_order) return MGP_OK;
  const int T = mgp_tile_side(c->g.N, c->np);
  if (!T) return mgp_set_error(MGP_EINVAL, "no tile side for Nmesh = %d", c->g.N);
  const int nt1 = c->g.N / T;
  const long long ntiles = (long long)nt1 * nt1 * nt1;
  c->tile_side = T;
  c->tile_n1 = nt1;
  const long long nblk = (ntiles + kScanChunk - 1) / kScanChunk;
  if (nblk > kScanChunk) return mgp_set_error(MGP_EINVAL, "%lld tiles exceed the scan's capacity", ntiles);
  MGP_CUDA(cudaMalloc(&c->tile_of, sizeof(unsigned) * (size_t)c->np));
  MGP_CUDA(cudaMalloc(&c->tile_order, sizeof(unsigned) * (size_t)c->np));
  MGP_CUDA(cudaMalloc(&c->tile_count, sizeof(unsigned) * (size_t)ntiles));
  MGP_CUDA(cudaMalloc(&c->tile_off, sizeof(unsigned) * (size_t)(ntiles + 1)));
  MGP_CUDA(cudaMalloc(&c->tile_cursor, sizeof(unsigned) * (size_t)ntiles));
  MGP_CUDA(cudaMalloc(&c->tile_bsum, sizeof(unsigned) * (size_t)nblk));
  return MGP_OK;
}

void mgp_tiles_free(mgp_ctx *c) {
  void *b[] = {c->tile_of, c->tile_order, c->tile_count, c->tile_off, c->tile_cursor, c->tile_bsum,
               c->q, c->q_alt, c->s_alt, c->v_alt, c->D1_alt, c->D2_alt};
  for (void *x : b)
    if (x) cudaFree(x);
  c->tile_of = c->tile_order = c->tile_count = c->tile_off = c->tile_cursor = c->tile_bsum = NULL;
  c->q = c->q_alt = NULL;
  c->s_alt = c->v_alt = c->D1_alt = c->D2_alt = NULL;
  c->tile_ready = 0;
  c->permuted = 0;
}

static void swap_arrays(mgp_ctx *c) {
  float *t;
  t = c->s; c->s = c->s_alt; c->s_alt = t;
  t = c->v; c->v = c->v_alt; c->v_alt = t;
  t = c->D1; c->D1 = c->D1_alt; c->D1_alt = t;
  t = c->D2; c->D2 = c->D2_alt; c->D2_alt = t;
}

// Permute the particle arrays into the order of the last mgp_tiles_sort
// (into the second buffers, then swap); q follows the particles.
int mgp_tiles_permute(mgp_ctx *c) {
  const size_t bytes = sizeof(float) * 3 * (size_t)c->np;
  if (!c->s_alt) {
    MGP_CUDA(cudaMalloc(&c->s_alt, bytes));
    MGP_CUDA(cudaMalloc(&c->v_alt, bytes));
    MGP_CUDA(cudaMalloc(&c->D1_alt, bytes));
    MGP_CUDA(cudaMalloc(&c->D2_alt, bytes));
    MGP_CUDA(cudaMalloc(&c->q, sizeof(unsigned) * (size_t)c->np));
    MGP_CUDA(cudaMalloc(&c->q_alt, sizeof(unsigned) * (size_t)c->np));
  }
  k_permute<<<mgp_blocks_for(c->np, 8), kThreads, 0, c->stream>>>(c->tile_order, c->np, c->s, c->v, c->D1, c->D2,
                                                                  c->permuted ? c->q : NULL, c->s_alt, c->v_alt,
                                                                  c->D1_alt, c->D2_alt, c->q_alt);
  MGP_CHECK_LAUNCH();
  g_kernel_launches++;
  swap_arrays(c);
  unsigned *t = c->q;
  c->q = c->q_alt;
  c->q_alt = t;
  c->permuted = 1;
  return MGP_OK;
}

int mgp_particles_canonical(mgp_ctx *c) {
  if (!c->permuted) return MGP_OK;
  k_unpermute<<<mgp_blocks_for(c->np, 8), kThreads, 0, c->stream>>>(c->np, c->s, c->v, c->D1, c->D2, c->q, c->s_alt,
                                                                    c->v_alt, c->D1_alt, c->D2_alt);
  MGP_CHECK_LAUNCH();
  g_kernel_launches++;
  swap_arrays(c);
  c->permuted = 0;
  c->tile_age = 0;
  return MGP_OK;
}

// Bucket the particles of a single box by tile (their current positions).
int mgp_tiles_sort(mgp_ctx *c) {
  int rc = mgp_tiles_alloc(c);
  if (rc != MGP_OK) return rc;
  const int N = c->g.N, Ns = c->Ns, T = c->tile_side, nt1 = c->tile_n1;
  const long long ntiles = (long long)nt1 * nt1 * nt1;
  const int ls = lattice_log2(Ns);
  const float scale = (float)(N / c->p.Box);
  int tshift = 0;
  while ((1 << tshift) < T) tshift++;
  const unsigned *qp = c->permuted ? c->q : NULL;
  MGP_CUDA(cudaMemsetAsync(c->tile_count, 0, sizeof(unsigned) * (size_t)ntiles, c->stream));
  const int nb = mgp_blocks_for(c->np, 8);
  if (ls >= 0)
    k_tile_key<true><<<nb, kThreads, 0, c->stream>>>(c->s, c->dstate, c->np, Ns, ls, N, scale, tshift, nt1, qp,
                                                     c->tile_of, c->tile_count);
  else
    k_tile_key<false><<<nb, kThreads, 0, c->stream>>>(c->s, c->dstate, c->np, Ns, ls, N, scale, tshift, nt1, qp,
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
                                                                        c->tile_bsum, (unsigned)c->np);
  MGP_CHECK_LAUNCH();
  g_kernel_launches++;
  k_tile_scatter<<<nb, kThreads, 0, c->stream>>>(c->tile_of, c->np, c->tile_cursor, c->tile_order);
  MGP_CHECK_LAUNCH();
  g_kernel_launches++;
  c->tile_ready = 1;
  return MGP_OK;
}

// Tile deposit onto a mesh pre-set to -1 (after mgp_tiles_sort; identity:
// the arrays were just permuted into the sort's order).
int mgp_cic_tiles(mgp_ctx *c, float wpar, int identity) {
  const unsigned *ord = identity ? NULL : c->tile_order, *qp = c->permuted ? c->q : NULL;
  const int N = c->g.N, Ns = c->Ns, T = c->tile_side, nt1 = c->tile_n1;
  const int ls = lattice_log2(Ns);
  const float scale = (float)(N / c->p.Box);
  const int nb = mgp_blocks_for((long long)nt1 * nt1 * nt1 * kThreads, 8);
  if (T == 16 && ls >= 0)
    k_cic_tiles<16, true><<<nb, kThreads, 0, c->stream>>>(c->s, c->dstate, c->np, Ns, ls, N, scale, wpar, c->rho,
                                                          c->g.P, c->tile_off, ord, qp, nt1);
  else if (T == 16)
    k_cic_tiles<16, false><<<nb, kThreads, 0, c->stream>>>(c->s, c->dstate, c->np, Ns, ls, N, scale, wpar, c->rho,
                                                           c->g.P, c->tile_off, ord, qp, nt1);
  else if (ls >= 0)
    k_cic_tiles<8, true><<<nb, kThreads, 0, c->stream>>>(c->s, c->dstate, c->np, Ns, ls, N, scale, wpar, c->rho,
                                                         c->g.P, c->tile_off, ord, qp, nt1);
  else
    k_cic_tiles<8, false><<<nb, kThreads, 0, c->stream>>>(c->s, c->dstate, c->np, Ns, ls, N, scale, wpar, c->rho,
                                                          c->g.P, c->tile_off, ord, qp, nt1);
  MGP_CHECK_LAUNCH();
  g_kernel_launches++;
  return MGP_OK;
}
