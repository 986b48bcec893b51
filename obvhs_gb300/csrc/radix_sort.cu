// radix_sort.cu -- see radix_sort.cuh.
//
// Onesweep-style LSD radix sort (8-bit digits):
//   k_rs_zero      clears the histograms and look-back words (unless the
//                  kernel that wrote the keys already did, radix_zero)
//   k_rs_hist      one read of the keys: a 256-bin histogram per digit; the
//                  last block turns them into global digit bases
//   k_rs_pass      per digit: tiles claimed in launch order rank their keys
//                  stably (warp match + per-warp digit counts), publish their
//                  digit counts and find their global offsets by decoupled
//                  look-back over earlier tiles, then reorder the tile by
//                  digit in shared memory and write each digit's run to
//                  consecutive addresses.
// No host synchronisation.  The look-back waits only on tiles that were
// claimed earlier and are therefore resident; every wait is bounded (the
// context's wait limit: empty look-back rounds a tile tolerates) and sets a
// status bit instead of spinning forever.  A tile that gives up still
// publishes an inclusive count (a partial one), so later tiles finish and
// every write stays inside the output; the caller checks the status before it
// uses the order.
#include "radix_sort.cuh"
#include "build.h"

namespace {

constexpr int THREADS = 256;
constexpr int WARPS = THREADS / 32;
constexpr uint32_t FLAG_AGG = 1u << 30;
constexpr uint32_t FLAG_INC = 2u << 30;
constexpr uint32_t VAL_MASK = (1u << 30) - 1;
constexpr int LB_WINDOW = 8;
constexpr int HIST_ITEMS = 8;

// Keys per thread: large sorts take big tiles (fewer tiles to look back
// over); small sorts take 4 per thread, so more tiles run at once and each
// tile's ranking chain is 4 rounds instead of 16.
constexpr uint32_t SMALL_SORT_MAX = 262144;
template <class K, bool SMALL>
struct Tile {
  static constexpr int ITEMS = SMALL ? 4 : (KeyTraits<K>::BYTES >= 16 ? 8 : 16);
  static constexpr int SIZE = THREADS * ITEMS;
};

// One tile of HIST_ITEMS keys per thread, all loads issued before the
// shared-memory counting, for the low `nd` digits.  The last block to finish
// (a ticket from `done`) turns every histogram into exclusive digit bases, so
// no separate scan launch is needed.
template <class K>
__global__ void __launch_bounds__(THREADS) k_rs_hist(const K* __restrict__ keys, uint32_t n, uint32_t* __restrict__ hist,
                                                     int nd, int first, uint32_t* done) {
  grid_dep_wait();
  constexpr int NB = KeyTraits<K>::BYTES;
  __shared__ uint32_t h[NB * 256];
  __shared__ uint32_t sw[WARPS];
  __shared__ bool s_last;
  for (int i = threadIdx.x; i < nd * 256; i += THREADS) h[i] = 0;
  const uint32_t base = blockIdx.x * (THREADS * HIST_ITEMS) + threadIdx.x;
  K k[HIST_ITEMS];
#pragma unroll
  for (int r = 0; r < HIST_ITEMS; r++)
    if (base + r * THREADS < n) k[r] = keys[base + r * THREADS];
  __syncthreads();
#pragma unroll
  for (int r = 0; r < HIST_ITEMS; r++)
    if (base + r * THREADS < n) {
#pragma unroll
      for (int b = 0; b < NB; b++)
        if (b < nd) atomicAdd(&h[b * 256 + KeyTraits<K>::digit(k[r], first + b)], 1u);
    }
  __syncthreads();
  for (int i = threadIdx.x; i < nd * 256; i += THREADS)
    if (h[i]) atomicAdd(&hist[i], h[i]);
  // release this block's counts, then take a ticket
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) s_last = atomicAdd(done, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int b = 0; b < nd; b++) {
    uint32_t* hb = hist + b * 256;
    const uint32_t v = __ldcg(&hb[threadIdx.x]);
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) sw[warp] = x;
    __syncthreads();
    uint32_t pre = 0;
    for (int w = 0; w < warp; w++) pre += sw[w];
    hb[threadIdx.x] = pre + x - v;
    __syncthreads();
  }
}

__global__ void k_rs_zero(uint4* p, size_t quads) {
  grid_dep_wait();
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < quads; i += (size_t)gridDim.x * blockDim.x)
    p[i] = make_uint4(0u, 0u, 0u, 0u);
}

// One digit pass.  Warp w of a tile owns the contiguous keys
// [w * 32 * ITEMS, (w + 1) * 32 * ITEMS) of the tile, so (warp, round, lane)
// is input order and each warp ranks its keys stably against its own digit
// histogram without block barriers; one scan over the warps' histograms per
// digit then gives every key its place in the tile.
template <class K, bool SMALL>
__global__ void __launch_bounds__(THREADS, 2) k_rs_pass(const K* __restrict__ keys_in, const uint32_t* __restrict__ vals_in,
                                                     K* __restrict__ keys_out, uint32_t* __restrict__ vals_out,
                                                     uint32_t n, int byte, bool iota,
                                                     const uint32_t* __restrict__ digit_base,
                                                     uint32_t* tile_status, uint32_t* tile_counter, uint32_t* status,
                                                     uint32_t spin_limit) {
  grid_dep_wait();
  constexpr int ITEMS = Tile<K, SMALL>::ITEMS;
  constexpr int TS = Tile<K, SMALL>::SIZE;
  __shared__ uint32_t s_tile;
  __shared__ uint32_t s_wh[WARPS][256];  // per-warp digit counts, then per-warp exclusive offsets
  __shared__ uint32_t s_off[256];        // global offset of each digit for this tile
  __shared__ uint32_t s_tloc[256];       // start of each digit inside the tile (tile-local order)
  __shared__ uint32_t s_wsum[WARPS];
  // the tile in digit order: keys, then (reusing the space) values, and each
  // slot's digit, so that the scatter writes consecutive addresses per digit
  __shared__ __align__(16) unsigned char s_stage[TS * (sizeof(K) > 4 ? sizeof(K) : 4)];
  __shared__ uint8_t s_dig[TS];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) s_tile = atomicAdd(tile_counter, 1u);
#pragma unroll
  for (int w = 0; w < WARPS; w++) s_wh[w][tid] = 0;
  __syncthreads();
  const uint32_t tile = s_tile;
  const uint32_t wbase = tile * TS + warp * 32 * ITEMS;
  const uint32_t lt_mask = (1u << lane) - 1u;
  K key[ITEMS];
  uint32_t val[ITEMS], rank[ITEMS];
#pragma unroll
  for (int r = 0; r < ITEMS; r++) {
    const uint32_t i = wbase + r * 32 + lane;
    if (i < n) {
      key[r] = keys_in[i];
      val[r] = iota ? i : vals_in[i];
    }
  }
  uint32_t* wh = s_wh[warp];
#pragma unroll
  for (int r = 0; r < ITEMS; r++) {
    const uint32_t i = wbase + r * 32 + lane;
    const bool valid = i < n;
    const uint32_t d = valid ? KeyTraits<K>::digit(key[r], byte) : 256u;
    const uint32_t peers = __match_any_sync(0xffffffffu, d);
    const uint32_t lrank = __popc(peers & lt_mask);
    const uint32_t before = valid ? wh[d] : 0u;
    __syncwarp();
    if (valid && lrank == 0) wh[d] = before + __popc(peers);
    __syncwarp();
    rank[r] = before + lrank;
  }
  __syncthreads();
  // per digit (thread tid): warp offsets inside the tile and the tile count
  uint32_t count = 0;
#pragma unroll
  for (int w = 0; w < WARPS; w++) {
    const uint32_t c = s_wh[w][tid];
    s_wh[w][tid] = count;
    count += c;
  }
  // exclusive scan of this tile's digit counts: the tile in digit order
  {
    uint32_t x = count;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) s_wsum[warp] = x;
    __syncthreads();
    uint32_t pre = 0;
#pragma unroll
    for (int w = 0; w < WARPS; w++)
      if (w < warp) pre += s_wsum[w];
    s_tloc[tid] = pre + x - count;
  }
  __syncthreads();
  // keys to shared memory in digit order (rank[r] becomes the tile position),
  // which frees their registers before the look-back
  K* sk = reinterpret_cast<K*>(s_stage);
#pragma unroll
  for (int r = 0; r < ITEMS; r++) {
    if (wbase + r * 32 + lane < n) {
      const uint32_t d = KeyTraits<K>::digit(key[r], byte);
      rank[r] += s_tloc[d] + wh[d];
      sk[rank[r]] = key[r];
      s_dig[rank[r]] = (uint8_t)d;
    }
  }
  // publish this tile's count of digit `tid`, then look back for the prefix,
  // LB_WINDOW earlier tiles per step (positions before tile 0 read as an
  // inclusive zero)
  uint32_t* my = tile_status + (size_t)tile * 256 + tid;
  uint32_t prefix = 0;
  if (tile == 0) {
    atomicExch(my, FLAG_INC | count);
  } else {
    atomicExch(my, FLAG_AGG | count);
    int64_t t = (int64_t)tile - 1;
    uint32_t spins = 0;
    for (;;) {
      uint32_t v[LB_WINDOW];
#pragma unroll
      for (int w = 0; w < LB_WINDOW; w++)
        v[w] = t - w >= 0 ? *((volatile uint32_t*)(tile_status + (size_t)(t - w) * 256 + tid)) : (uint32_t)FLAG_INC;
      bool stop = false, blocked = false;
      int adv = 0;
#pragma unroll
      for (int w = 0; w < LB_WINDOW; w++) {
        if (stop || blocked) continue;
        if ((v[w] & ~VAL_MASK) == 0) {
          blocked = true;
        } else {
          prefix += v[w] & VAL_MASK;
          adv++;
          stop = (v[w] & FLAG_INC) != 0;
        }
      }
      if (stop) break;
      t -= adv;
      if (adv == 0 && ++spins > spin_limit) {
        atomicOr(status, 4u);  // ST_ITER_LIMIT
        break;
      }
    }
    atomicExch(my, FLAG_INC | (prefix + count));
  }
  s_off[tid] = digit_base[tid] + prefix;
  __syncthreads();
  // each digit's run of the tile to consecutive addresses
  const uint32_t tile_n = min((uint32_t)TS, n - tile * TS);
  for (uint32_t j = tid; j < tile_n; j += THREADS) {
    const uint32_t d = s_dig[j];
    keys_out[s_off[d] + (j - s_tloc[d])] = sk[j];
  }
  __syncthreads();
  uint32_t* sv = reinterpret_cast<uint32_t*>(s_stage);
#pragma unroll
  for (int r = 0; r < ITEMS; r++)
    if (wbase + r * 32 + lane < n) sv[rank[r]] = val[r];
  __syncthreads();
  for (uint32_t j = tid; j < tile_n; j += THREADS) {
    const uint32_t d = s_dig[j];
    vals_out[s_off[d] + (j - s_tloc[d])] = sv[j];
  }
}

__global__ void k_iota(uint32_t* v, uint32_t n) {
  grid_dep_wait();
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) v[i] = i;
}

}  // namespace

uint32_t radix_tile_count(uint32_t n) { return (n + 1023) / 1024; }  // the smallest tile

size_t radix_scratch_words(uint32_t n) {
  // 16 histograms of 256 + per pass: tile status (256 per tile) + counter
  return 16 * 256 + 16 * ((size_t)radix_tile_count(n) * 256 + 32);
}

template <class K>
static uint32_t sort_tiles(uint32_t n) {
  const int TS = n <= SMALL_SORT_MAX ? Tile<K, true>::SIZE : Tile<K, false>::SIZE;
  return (n + TS - 1) / TS;
}

template <class K>
size_t radix_zero_words(uint32_t n, int digits) {
  constexpr int NB = KeyTraits<K>::BYTES;
  const int nd = digits > 0 && digits < NB ? digits : NB;
  return 16 * 256 + (size_t)nd * ((size_t)sort_tiles<K>(n) * 256 + 32);
}

template <class K>
cudaError_t radix_sort_pairs(obvhs_ctx& c, K* keys, uint32_t* vals, uint32_t n, bool init_iota, K* keys_alt,
                             uint32_t* vals_alt, uint32_t* scratch, bool* result_in_alt, int digits, bool zeroed,
                             const uint32_t* bases, int first_byte) {
  constexpr int NB = KeyTraits<K>::BYTES;
  const int nd = digits > 0 && digits < NB ? digits : NB;
  if (first_byte < 0 || first_byte + nd > NB) return cudaErrorInvalidValue;
  const bool small = n <= SMALL_SORT_MAX;
  *result_in_alt = false;
  if (n == 0) return cudaSuccess;
  const uint32_t ntiles = sort_tiles<K>(n);
  uint32_t* hist = scratch;
  uint32_t* pass_area = scratch + 16 * 256;
  const size_t pass_words = (size_t)ntiles * 256 + 32;
  if (!zeroed) {
    const size_t quads = radix_zero_words<K>(n, digits) / 4;
    const size_t cap = c.num_sms > 0 ? (size_t)c.num_sms * 8 : 1024;  // a bare context may not know its SMs
    const uint32_t zb = (uint32_t)std::min<size_t>((quads + 255) / 256, cap);
    KLAUNCH("k_rs_zero", launch_k(k_rs_zero, zb, 256, 0, c.stream, reinterpret_cast<uint4*>(scratch), quads));
  }
  if (bases) {
    hist = const_cast<uint32_t*>(bases);
  } else {
    const uint32_t hb = (n + THREADS * HIST_ITEMS - 1) / (THREADS * HIST_ITEMS);
    // pass 0's header word 1 is the histogram kernel's ticket counter
    KLAUNCH("k_rs_hist", launch_k(k_rs_hist<K>, hb, THREADS, 0, c.stream, keys, n, hist, nd, first_byte, pass_area + 1));
  }
  K* kin = keys;
  uint32_t* vin = vals;
  K* kout = keys_alt;
  uint32_t* vout = vals_alt;
  bool iota = init_iota;
  for (int b = 0; b < nd; b++) {
    uint32_t* ts = pass_area + (size_t)b * pass_words;
    if (small)
      KLAUNCH("k_rs_pass", launch_k(k_rs_pass<K, true>, ntiles, THREADS, 0, c.stream, kin, vin, kout, vout, n, first_byte + b, iota,
                                                                               hist + b * 256, ts + 32, ts, c.d_status,
                                                                               c.wait_limit));
    else
      KLAUNCH("k_rs_pass", launch_k(k_rs_pass<K, false>, ntiles, THREADS, 0, c.stream, kin, vin, kout, vout, n, first_byte + b, iota,
                                                                                hist + b * 256, ts + 32, ts, c.d_status,
                                                                               c.wait_limit));
    iota = false;
    std::swap(kin, kout);
    std::swap(vin, vout);
    *result_in_alt = !*result_in_alt;
  }
  return cudaGetLastError();
}

cudaError_t fill_iota(uint32_t* v, uint32_t n, cudaStream_t s) {
  if (!n) return cudaSuccess;
  uint32_t blocks = (n + 255) / 256;
  if (blocks > 4096) blocks = 4096;
  launch_k(k_iota, blocks, 256, 0, s, v, n);
  return cudaGetLastError();
}

template cudaError_t radix_sort_pairs<uint32_t>(obvhs_ctx&, uint32_t*, uint32_t*, uint32_t, bool, uint32_t*, uint32_t*,
                                                uint32_t*, bool*, int, bool, const uint32_t*, int);
template cudaError_t radix_sort_pairs<unsigned long long>(obvhs_ctx&, unsigned long long*, uint32_t*, uint32_t, bool,
                                                          unsigned long long*, uint32_t*, uint32_t*, bool*, int, bool,
                                                          const uint32_t*, int);
template cudaError_t radix_sort_pairs<U128>(obvhs_ctx&, U128*, uint32_t*, uint32_t, bool, U128*, uint32_t*, uint32_t*,
                                            bool*, int, bool, const uint32_t*, int);
template size_t radix_zero_words<uint32_t>(uint32_t, int);
template size_t radix_zero_words<unsigned long long>(uint32_t, int);
template size_t radix_zero_words<U128>(uint32_t, int);
