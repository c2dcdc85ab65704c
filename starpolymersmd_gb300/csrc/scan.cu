// Counting-sort support: exclusive prefix sum of the per-cell counts and the
// scatter that turns (cell, rank) keys into a cell-ordered permutation. This
// replaces MPC::sort's vector<vector<MPCParticle*>> push_back cell lists
// (star-polymers/lib/Hydrodynamics/MPC.cpp:201-237) with integer arithmetic.
//
// Scan: three launches over C cells: per-tile scan (2048 cells / CTA, count
// is re-zeroed for the next collision while it is read), scan of the tile
// totals (one CTA), add of the tile bases. off[C] receives the total.
#include <stdint.h>

#include "launch.h"
#include "mpc_kernels.cuh"

namespace smpc {

constexpr int SCAN_NT = 256;
constexpr int SCAN_IPT = 8;
constexpr int SCAN_TILE = SCAN_NT * SCAN_IPT;

__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* total) {
  __shared__ uint32_t warp_sums[SCAN_NT / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_sums[w] = x;
  __syncthreads();
  if (w == 0) {
    uint32_t s = lane < SCAN_NT / 32 ? warp_sums[lane] : 0u;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, s, o);
      if (lane >= o) s += y;
    }
    if (lane < SCAN_NT / 32) warp_sums[lane] = s;
  }
  __syncthreads();
  const uint32_t before = (w > 0 ? warp_sums[w - 1] : 0u) + x - v;
  *total = warp_sums[SCAN_NT / 32 - 1];
  return before;
}

// One tile of SCAN_TILE cells per CTA. Warp w owns the tile's w-th run of
// 32 * SCAN_IPT consecutive cells, read as SCAN_IPT rows of 32 (every load and
// store of a warp is one contiguous 128-byte row); each row is a warp scan
// carried into the next, then the warps' totals give each warp's base.
__global__ void __launch_bounds__(SCAN_NT) k_scan_tiles(uint32_t* __restrict__ count,
                                                        uint32_t* __restrict__ off,
                                                        uint32_t* __restrict__ tile_sum, int n) {
  __shared__ uint32_t warp_tot[SCAN_NT / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int seg = blockIdx.x * SCAN_TILE + w * (32 * SCAN_IPT);
  uint32_t c[SCAN_IPT], pre[SCAN_IPT];
#pragma unroll
  for (int k = 0; k < SCAN_IPT; ++k) {
    const int i = seg + 32 * k + lane;
    c[k] = i < n ? count[i] : 0u;
  }
#pragma unroll
  for (int k = 0; k < SCAN_IPT; ++k) {
    const int i = seg + 32 * k + lane;
    if (i < n) count[i] = 0u;  // re-zeroed for the next collision
  }
  uint32_t carry = 0;
#pragma unroll
  for (int k = 0; k < SCAN_IPT; ++k) {
    uint32_t x = c[k];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
      if (lane >= o) x += y;
    }
    pre[k] = carry + x - c[k];
    carry += __shfl_sync(0xFFFFFFFFu, x, 31);
  }
  if (lane == 0) warp_tot[w] = carry;
  __syncthreads();
  uint32_t wbase = 0, total = 0;
#pragma unroll
  for (int q = 0; q < SCAN_NT / 32; ++q) {
    const uint32_t t = warp_tot[q];
    if (q < w) wbase += t;
    total += t;
  }
#pragma unroll
  for (int k = 0; k < SCAN_IPT; ++k) {
    const int i = seg + 32 * k + lane;
    if (i < n) off[i] = wbase + pre[k];
  }
  if (threadIdx.x == 0) tile_sum[blockIdx.x] = total;
}

// Exclusive scan of up to SCAN_TILE tile totals in one CTA.
__global__ void __launch_bounds__(SCAN_NT) k_scan_tile_sums(uint32_t* __restrict__ tile_sum,
                                                            int n_tiles,
                                                            uint32_t* __restrict__ grand) {
  uint32_t carry = 0;
  for (int chunk = 0; chunk < n_tiles; chunk += SCAN_TILE) {
    const int base = chunk + threadIdx.x * SCAN_IPT;
    uint32_t c[SCAN_IPT];
    uint32_t s = 0;
#pragma unroll
    for (int k = 0; k < SCAN_IPT; ++k) {
      c[k] = base + k < n_tiles ? tile_sum[base + k] : 0u;
      s += c[k];
    }
    uint32_t total;
    uint32_t run = block_exclusive_scan(s, &total) + carry;
#pragma unroll
    for (int k = 0; k < SCAN_IPT; ++k) {
      if (base + k < n_tiles) tile_sum[base + k] = run;
      run += c[k];
    }
    carry += total;
    __syncthreads();
  }
  if (threadIdx.x == 0) *grand = carry;
}

// SCAN_ADD_U cells per thread, a block apart (coalesced, independent loads)
constexpr int SCAN_ADD_U = 4;
__global__ void __launch_bounds__(SCAN_NT) k_scan_add(uint32_t* __restrict__ off,
                                                      const uint32_t* __restrict__ tile_base,
                                                      const uint32_t* __restrict__ grand, int n) {
  const int base = blockIdx.x * (SCAN_NT * SCAN_ADD_U) + threadIdx.x;
  uint32_t v[SCAN_ADD_U];
#pragma unroll
  for (int u = 0; u < SCAN_ADD_U; ++u) {
    const int i = base + u * SCAN_NT;
    v[u] = i < n ? off[i] + tile_base[i / SCAN_TILE] : 0u;
  }
#pragma unroll
  for (int u = 0; u < SCAN_ADD_U; ++u) {
    const int i = base + u * SCAN_NT;
    if (i < n) off[i] = v[u];
    if (i == n) off[n] = *grand;
  }
}

// perm[off[cell] + rank] = source. Each thread takes PERM_U entries a block
// apart and issues all key loads, then all offset gathers, then the stores,
// so PERM_U independent gather chains are in flight per thread. A position
// past the last entry (counts that do not match the keys; never expected) is
// reported in the error word, not written.
constexpr int PERM_NT = 256;
constexpr int PERM_U = 4;
__global__ void __launch_bounds__(PERM_NT) k_build_perm(const uint2* __restrict__ keys, int n_slots,
                                                        const uint2* __restrict__ mkey, int n_mono,
                                                        const uint32_t* __restrict__ off,
                                                        uint32_t* __restrict__ perm,
                                                        ErrorState* err) {
  const int n = n_slots + n_mono;
  const int base = blockIdx.x * (PERM_NT * PERM_U) + threadIdx.x;
  uint2 k[PERM_U];
#pragma unroll
  for (int u = 0; u < PERM_U; ++u) {
    const int i = base + u * PERM_NT;
    k[u] = make_uint2(KEY_NONE, 0u);
    if (i < n_slots)
      k[u] = keys[i];
    else if (i < n)
      k[u] = mkey[i - n_slots];
  }
  uint32_t o[PERM_U];
#pragma unroll
  for (int u = 0; u < PERM_U; ++u) o[u] = k[u].x != KEY_NONE ? off[k[u].x] : 0u;
#pragma unroll
  for (int u = 0; u < PERM_U; ++u) {
    const int i = base + u * PERM_NT;
    if (k[u].x == KEY_NONE) continue;
    const uint32_t pos = o[u] + k[u].y;
    if (pos < static_cast<uint32_t>(n))
      perm[pos] = i < n_slots ? static_cast<uint32_t>(i) : (MONO_BIT | static_cast<uint32_t>(i - n_slots));
    else
      raise_error(err, ERR_KEY_MISMATCH, pos, k[u].x);
  }
}

// The same scatter from packed solvent keys (local cell << 16 | rank, written
// by the packed binning): one block per binning tile of slots, whose replica
// gives the cell base; the monomers' (global cell, rank) keys in the blocks
// after the tiles.
__global__ void __launch_bounds__(PERM_NT) k_build_perm_packed(
    const Tile* tiles, int n_tiles, const RepInfo* reps, const uint32_t* __restrict__ keys,
    int n_slots, const uint2* __restrict__ mkey, int n_mono, const uint32_t* __restrict__ off,
    uint32_t* __restrict__ perm, ErrorState* err) {
  const uint32_t n = static_cast<uint32_t>(n_slots + n_mono);
  if (static_cast<int>(blockIdx.x) < n_tiles) {
    const Tile t = tiles[blockIdx.x];
    const uint32_t cbase = static_cast<uint32_t>(reps[t.rep].cell_base);
    for (int base = t.begin + static_cast<int>(threadIdx.x); base < t.end;
         base += PERM_NT * PERM_U) {
      uint32_t k[PERM_U], o[PERM_U];
#pragma unroll
      for (int u = 0; u < PERM_U; ++u) {
        const int i = base + u * PERM_NT;
        k[u] = i < t.end ? keys[i] : KEY_NONE;
      }
#pragma unroll
      for (int u = 0; u < PERM_U; ++u) o[u] = k[u] != KEY_NONE ? off[cbase + (k[u] >> 16)] : 0u;
#pragma unroll
      for (int u = 0; u < PERM_U; ++u) {
        if (k[u] == KEY_NONE) continue;
        const uint32_t pos = o[u] + (k[u] & 0xFFFFu);
        if (pos < n)
          perm[pos] = static_cast<uint32_t>(base + u * PERM_NT);
        else
          raise_error(err, ERR_KEY_MISMATCH, pos, k[u]);
      }
    }
    return;
  }
  const int base = (static_cast<int>(blockIdx.x) - n_tiles) * (PERM_NT * PERM_U) +
                   static_cast<int>(threadIdx.x);
#pragma unroll
  for (int u = 0; u < PERM_U; ++u) {
    const int i = base + u * PERM_NT;
    if (i >= n_mono) continue;
    const uint2 k = mkey[i];
    if (k.x == KEY_NONE) continue;
    const uint32_t pos = off[k.x] + k.y;
    if (pos < n)
      perm[pos] = MONO_BIT | static_cast<uint32_t>(i);
    else
      raise_error(err, ERR_KEY_MISMATCH, pos, k.x);
  }
}

int scan_tile_count(int n_cells) { return (n_cells + SCAN_TILE - 1) / SCAN_TILE; }

void launch_scan(uint32_t* count, uint32_t* off, uint32_t* tile_sum, uint32_t* grand,
                 int n_cells, cudaStream_t st) {
  const int tiles = scan_tile_count(n_cells);
  k_scan_tiles<<<tiles, SCAN_NT, 0, st>>>(count, off, tile_sum, n_cells);
  k_scan_tile_sums<<<1, SCAN_NT, 0, st>>>(tile_sum, tiles, grand);
  const int per_block = SCAN_NT * SCAN_ADD_U;
  k_scan_add<<<(n_cells + 1 + per_block - 1) / per_block, SCAN_NT, 0, st>>>(off, tile_sum, grand,
                                                                           n_cells);
}

void launch_build_perm_packed(const Tile* tiles, int n_tiles, const RepInfo* reps,
                              const uint32_t* keys, int n_slots, const uint2* mkey, int n_mono,
                              const uint32_t* off, uint32_t* perm, ErrorState* err,
                              cudaStream_t st) {
  const int mono_blocks = (n_mono + PERM_NT * PERM_U - 1) / (PERM_NT * PERM_U);
  if (n_tiles + mono_blocks == 0) return;
  k_build_perm_packed<<<n_tiles + mono_blocks, PERM_NT, 0, st>>>(tiles, n_tiles, reps, keys,
                                                                 n_slots, mkey, n_mono, off, perm,
                                                                 err);
}

void launch_build_perm(const uint2* keys, int n_slots, const uint2* mkey, int n_mono,
                       const uint32_t* off, uint32_t* perm, ErrorState* err, cudaStream_t st) {
  const int n = n_slots + n_mono;
  if (n == 0) return;
  k_build_perm<<<(n + PERM_NT * PERM_U - 1) / (PERM_NT * PERM_U), PERM_NT, 0, st>>>(
      keys, n_slots, mkey, n_mono, off, perm, err);
}

}  // namespace smpc
