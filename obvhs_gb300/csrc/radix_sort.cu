// radix_sort.cu -- see radix_sort.cuh.
#include "radix_sort.cuh"

namespace {

constexpr int THREADS = 256;
constexpr int ROUNDS = RADIX_TILE / THREADS;  // 16
constexpr int WARPS = THREADS / 32;

template <class K>
__global__ void __launch_bounds__(THREADS) k_rs_hist_all(const K* __restrict__ keys, uint32_t n,
                                                         uint32_t* __restrict__ all_hist) {
  constexpr int NB = KeyTraits<K>::BYTES;
  __shared__ uint32_t h[NB * 256];
  for (int i = threadIdx.x; i < NB * 256; i += THREADS) h[i] = 0;
  __syncthreads();
  for (uint32_t i = blockIdx.x * THREADS + threadIdx.x; i < n; i += gridDim.x * THREADS) {
    K k = keys[i];
#pragma unroll
    for (int b = 0; b < NB; b++) atomicAdd(&h[b * 256 + KeyTraits<K>::digit(k, b)], 1u);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < NB * 256; i += THREADS)
    if (h[i]) atomicAdd(&all_hist[i], h[i]);
}

template <class K>
__global__ void __launch_bounds__(THREADS) k_rs_tile_hist(const K* __restrict__ keys, uint32_t n, int byte,
                                                          uint32_t ntiles, uint32_t* __restrict__ tile_hist) {
  __shared__ uint32_t h[256];
  h[threadIdx.x] = 0;
  __syncthreads();
  uint32_t base = blockIdx.x * RADIX_TILE;
#pragma unroll 4
  for (int r = 0; r < ROUNDS; r++) {
    uint32_t i = base + r * THREADS + threadIdx.x;
    if (i < n) atomicAdd(&h[KeyTraits<K>::digit(keys[i], byte)], 1u);
  }
  __syncthreads();
  tile_hist[threadIdx.x * ntiles + blockIdx.x] = h[threadIdx.x];
}

// One block per digit: exclusive scan of its tile counts, offset by the
// number of keys with a smaller digit.
__global__ void __launch_bounds__(THREADS) k_rs_tile_scan(uint32_t* __restrict__ tile_hist, uint32_t ntiles,
                                                          const uint32_t* __restrict__ digit_hist) {
  __shared__ uint32_t s_base;
  __shared__ uint32_t s_warp[WARPS];
  const uint32_t d = blockIdx.x;
  if (threadIdx.x == 0) {
    uint32_t b = 0;
    for (uint32_t k = 0; k < d; k++) b += digit_hist[k];
    s_base = b;
  }
  __syncthreads();
  uint32_t carry = s_base;
  uint32_t* row = tile_hist + (size_t)d * ntiles;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (uint32_t start = 0; start < ntiles; start += THREADS) {
    uint32_t t = start + threadIdx.x;
    uint32_t v = t < ntiles ? row[t] : 0;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    uint32_t wp = 0, tot = 0;
    for (int w = 0; w < WARPS; w++) {
      uint32_t c = s_warp[w];
      if (w < warp) wp += c;
      tot += c;
    }
    if (t < ntiles) row[t] = carry + wp + x - v;
    carry += tot;
    __syncthreads();
  }
}

template <class K>
__global__ void __launch_bounds__(THREADS) k_rs_scatter(const K* __restrict__ keys_in, const uint32_t* __restrict__ vals_in,
                                                        K* __restrict__ keys_out, uint32_t* __restrict__ vals_out,
                                                        uint32_t n, int byte, uint32_t ntiles,
                                                        const uint32_t* __restrict__ tile_off, bool iota) {
  __shared__ uint32_t s_off[256];
  __shared__ uint32_t s_cnt[WARPS][256];
  __shared__ uint32_t s_pre[WARPS][256];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  s_off[tid] = tile_off[(size_t)tid * ntiles + blockIdx.x];
#pragma unroll
  for (int w = 0; w < WARPS; w++) s_cnt[w][tid] = 0;
  __syncthreads();
  const uint32_t lt_mask = (1u << lane) - 1u;
  uint32_t base = blockIdx.x * RADIX_TILE;
  for (int r = 0; r < ROUNDS; r++) {
    uint32_t i = base + r * THREADS + tid;
    bool valid = i < n;
    K k;
    uint32_t v = 0, d = 256;
    if (valid) {
      k = keys_in[i];
      v = iota ? i : vals_in[i];
      d = KeyTraits<K>::digit(k, byte);
    }
    uint32_t peers = __match_any_sync(0xffffffffu, d);
    uint32_t lrank = __popc(peers & lt_mask);
    if (valid && lrank == 0) s_cnt[warp][d] = __popc(peers);
    __syncthreads();
    {
      uint32_t run = s_off[tid];
#pragma unroll
      for (int w = 0; w < WARPS; w++) {
        uint32_t c = s_cnt[w][tid];
        s_pre[w][tid] = run;
        s_cnt[w][tid] = 0;
        run += c;
      }
      s_off[tid] = run;
    }
    __syncthreads();
    if (valid) {
      uint32_t pos = s_pre[warp][d] + lrank;
      keys_out[pos] = k;
      vals_out[pos] = v;
    }
  }
}

}  // namespace

uint32_t radix_tile_count(uint32_t n) { return (n + RADIX_TILE - 1) / RADIX_TILE; }

template <class K>
cudaError_t radix_sort_pairs(K* keys, uint32_t* vals, uint32_t n, bool init_iota, K* keys_alt, uint32_t* vals_alt,
                             uint32_t* tile_hist, uint32_t* all_hist, uint32_t* h_all_hist, cudaStream_t stream,
                             bool* result_in_alt, uint64_t* launches) {
  constexpr int NB = KeyTraits<K>::BYTES;
  *result_in_alt = false;
  if (n == 0) return cudaSuccess;
  cudaError_t e = cudaMemsetAsync(all_hist, 0, NB * 256 * sizeof(uint32_t), stream);
  if (e) return e;
  uint32_t hist_blocks = (n + THREADS * 16 - 1) / (THREADS * 16);
  if (hist_blocks > 1024) hist_blocks = 1024;
  k_rs_hist_all<K><<<hist_blocks, THREADS, 0, stream>>>(keys, n, all_hist);
  *launches += 1;
  e = cudaMemcpyAsync(h_all_hist, all_hist, NB * 256 * sizeof(uint32_t), cudaMemcpyDeviceToHost, stream);
  if (e) return e;
  e = cudaStreamSynchronize(stream);
  if (e) return e;
  uint32_t ntiles = radix_tile_count(n);
  K* kin = keys;
  uint32_t* vin = vals;
  K* kout = keys_alt;
  uint32_t* vout = vals_alt;
  bool iota = init_iota;
  for (int b = 0; b < NB; b++) {
    bool constant = false;
    for (int d = 0; d < 256; d++)
      if (h_all_hist[b * 256 + d] == n) constant = true;
    if (constant) continue;
    k_rs_tile_hist<K><<<ntiles, THREADS, 0, stream>>>(kin, n, b, ntiles, tile_hist);
    k_rs_tile_scan<<<256, THREADS, 0, stream>>>(tile_hist, ntiles, all_hist + b * 256);
    k_rs_scatter<K><<<ntiles, THREADS, 0, stream>>>(kin, vin, kout, vout, n, b, ntiles, tile_hist, iota);
    *launches += 3;
    iota = false;
    K* tk = kin;
    kin = kout;
    kout = tk;
    uint32_t* tv = vin;
    vin = vout;
    vout = tv;
    *result_in_alt = !*result_in_alt;
  }
  if (iota) {
    // every digit was constant: the order is the identity
    extern cudaError_t fill_iota(uint32_t*, uint32_t, cudaStream_t);
    e = fill_iota(vals, n, stream);
    *launches += 1;
    if (e) return e;
  }
  return cudaGetLastError();
}

namespace {
__global__ void k_iota(uint32_t* v, uint32_t n) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) v[i] = i;
}
}  // namespace

cudaError_t fill_iota(uint32_t* v, uint32_t n, cudaStream_t s) {
  if (!n) return cudaSuccess;
  uint32_t blocks = (n + 255) / 256;
  if (blocks > 4096) blocks = 4096;
  k_iota<<<blocks, 256, 0, s>>>(v, n);
  return cudaGetLastError();
}

template cudaError_t radix_sort_pairs<uint32_t>(uint32_t*, uint32_t*, uint32_t, bool, uint32_t*, uint32_t*, uint32_t*,
                                                uint32_t*, uint32_t*, cudaStream_t, bool*, uint64_t*);
template cudaError_t radix_sort_pairs<unsigned long long>(unsigned long long*, uint32_t*, uint32_t, bool,
                                                          unsigned long long*, uint32_t*, uint32_t*, uint32_t*,
                                                          uint32_t*, cudaStream_t, bool*, uint64_t*);
template cudaError_t radix_sort_pairs<U128>(U128*, uint32_t*, uint32_t, bool, U128*, uint32_t*, uint32_t*, uint32_t*,
                                            uint32_t*, cudaStream_t, bool*, uint64_t*);
