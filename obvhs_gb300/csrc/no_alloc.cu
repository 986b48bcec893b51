// no_alloc.cu -- obvhs_morton_sort_noalloc: the Morton-code sort of
// obvhs_morton_sort for callers that cannot allocate device memory.
//
// Who needs it: a renderer or engine that reserves the GPU's memory up front
// in its own pool (so a cudaMalloc from this library would fail, or would
// fragment memory the caller manages), and frame-time code on which the
// device-wide synchronisation that cudaMalloc/cudaFree can cause is not
// acceptable.  Such callers hand over device buffers for the inputs and the
// outputs; everything else the sort needs lives in one fixed scratch array
// that is part of this library's device image.
//
// The scratch array: a file-scope __device__ array of NOALLOC_SCRATCH_BYTES
// (about 22 MiB, enough for OBVHS_NOALLOC_MAX_PRIMS primitives).  Every GPU on
// which this entry point runs holds it until the process exits; under eager
// module loading (CUDA_MODULE_LOADING=EAGER) every GPU that uses this library
// at all holds it, whether or not this entry point is called.  On the host,
// `g_noalloc_scratch` only names the symbol; its device address comes from
// cudaGetSymbolAddress, taken once per device (with that device current) by
// the first call on that device, which is why that first call should come
// before any stream capture.  The address is kept for the life of the
// process: after cudaDeviceReset on a device this entry point must not be
// called on that device again.
//
// Sharing: every call on a device uses the same array, and the array keeps
// what the last call left there.  Each call therefore re-initialises what must
// start at zero or at a known value (status word, scene bounds, radix
// histograms and look-back words); the rest is overwritten before it is read.
// Two calls whose work overlaps on the GPU (different streams, or different
// host threads on one device) race on the array and corrupt each other:
// serialise them.
//
// This entry point calls no cudaMalloc, cudaFree or allocating library
// routine.  It launches the same kernels as obvhs_morton_sort (leaf boxes,
// Morton codes, radix sort) with pointers into the scratch array, plus two
// copy kernels into the caller's outputs, then synchronises the caller's
// stream to read the status word.
#include <mutex>

#include "build.h"
#include "radix_sort.cuh"

namespace {

constexpr uint32_t MAX_PRIMS = OBVHS_NOALLOC_MAX_PRIMS;

constexpr size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// Byte layout of the scratch array (each region starts on 256 bytes).
constexpr size_t OFF_STATUS = 0;                                           // u32 status word
constexpr size_t OFF_TOTAL = 256;                                          // int[6] scene bound keys
constexpr size_t OFF_LEAVES = 512;                                         // Bvh2Node[MAX_PRIMS]
constexpr size_t OFF_KEYS = align256(OFF_LEAVES + (size_t)MAX_PRIMS * sizeof(Bvh2Node));  // U128 or u64 keys
constexpr size_t OFF_KEYS_ALT = align256(OFF_KEYS + (size_t)MAX_PRIMS * sizeof(U128));
constexpr size_t OFF_VALS = align256(OFF_KEYS_ALT + (size_t)MAX_PRIMS * sizeof(U128));
constexpr size_t OFF_VALS_ALT = align256(OFF_VALS + (size_t)MAX_PRIMS * 4);
constexpr size_t OFF_RADIX = align256(OFF_VALS_ALT + (size_t)MAX_PRIMS * 4);
// radix_scratch_words(n) = 16 histograms of 256 words + 16 passes of
// (tiles of 1024 keys (the smallest tile) x 256 words + 32); checked against
// the real function
// when a device is set up.
constexpr size_t RADIX_WORDS = 16 * 256 + 16 * ((size_t)((MAX_PRIMS + 1023) / 1024) * 256 + 32);
constexpr size_t NOALLOC_SCRATCH_BYTES = align256(OFF_RADIX + RADIX_WORDS * 4);

constexpr int MAX_DEVICES = 64;

__device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];

std::mutex g_setup_mutex;
unsigned char* g_scratch_ptr[MAX_DEVICES] = {};

// Device address of the scratch array on the current device `dev`; the first
// call per device looks it up.  Returns a cudaError_t.
cudaError_t scratch_on_device(int dev, unsigned char** out) {
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_ptr[dev]) {
    unsigned char* ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress((void**)&ptr, g_noalloc_scratch);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return e;
    }
    g_scratch_ptr[dev] = ptr;
  }
  *out = g_scratch_ptr[dev];
  return cudaSuccess;
}

// True when p is device memory of device `dev` (the current device) or
// managed memory.  Device memory of another GPU is rejected: the kernels run
// on `dev` and would reach it only through peer access, which this entry
// point does not set up.
bool on_device(const void* p, int dev) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  if (a.type == cudaMemoryTypeManaged) return true;
  return a.type == cudaMemoryTypeDevice && a.device == dev;
}

// Codes in the layout obvhs_morton_sort returns: (lo, hi) u64 pairs.
__global__ void k_codes_out(const unsigned long long* __restrict__ keys, uint32_t n, int precision,
                            unsigned long long* __restrict__ codes) {
  grid_dep_wait();
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    codes[2 * (size_t)i] = precision ? keys[2 * (size_t)i] : keys[i];
    codes[2 * (size_t)i + 1] = precision ? keys[2 * (size_t)i + 1] : 0ull;
  }
}

__global__ void k_order_out(const uint32_t* __restrict__ src, uint32_t n, uint32_t* __restrict__ order) {
  grid_dep_wait();
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) order[i] = src[i];
}

}  // namespace

extern "C" {

OBVHS_API int obvhs_morton_sort_noalloc(const float* aabbs, uint32_t n, uint32_t sort_precision, uint64_t* codes,
                                        uint32_t* order, void* stream) {
  if (n > MAX_PRIMS) return OBVHS_ERR_TOO_LARGE;
  if (sort_precision > 1) return OBVHS_ERR_INVALID_ARG;
  if (n == 0) return OBVHS_OK;
  if (!aabbs || !order) return OBVHS_ERR_INVALID_ARG;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAX_DEVICES) {
    cudaGetLastError();
    return OBVHS_ERR_CUDA;
  }
  if (!on_device(aabbs, dev) || !on_device(order, dev) || (codes && !on_device(codes, dev)))
    return OBVHS_ERR_INVALID_ARG;
  if (radix_scratch_words(MAX_PRIMS) > RADIX_WORDS) return OBVHS_ERR_INVALID_ARG;
  unsigned char* base = nullptr;
  if (scratch_on_device(dev, &base) != cudaSuccess) return OBVHS_ERR_CUDA;

  // A context on the stack carries the caller's stream and the status word;
  // its scratch pool stays empty and is never used.
  obvhs_ctx c;
  c.device = dev;
  if (cudaDeviceGetAttribute(&c.num_sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
    cudaGetLastError();
    return OBVHS_ERR_CUDA;
  }
  c.stream = (cudaStream_t)stream;
  c.d_status = (uint32_t*)(base + OFF_STATUS);
  Bvh2Node* leaves = (Bvh2Node*)(base + OFF_LEAVES);
  int* total = (int*)(base + OFF_TOTAL);
  void* keys = base + OFF_KEYS;
  void* keys_alt = base + OFF_KEYS_ALT;
  uint32_t* vals = (uint32_t*)(base + OFF_VALS);
  uint32_t* vals_alt = (uint32_t*)(base + OFF_VALS_ALT);
  uint32_t* rs = (uint32_t*)(base + OFF_RADIX);

  if (cudaMemsetAsync(c.d_status, 0, 4, c.stream) != cudaSuccess) {
    cudaGetLastError();
    return OBVHS_ERR_CUDA;
  }
  int r = ploc_leaves(c, nullptr, aabbs, nullptr, n, leaves, total);
  if (!r) r = ploc_morton_codes(c, leaves, n, total, (int)sort_precision, keys);
  if (r) return r;
  const uint32_t g = div_up<uint32_t>(n, 256) < 4096 ? div_up<uint32_t>(n, 256) : 4096;
  if (codes)  // codes in input order, before the sort reorders them
    launch_k(k_codes_out, g, 256, 0, c.stream, (const unsigned long long*)keys, n, (int)sort_precision,
                                         (unsigned long long*)codes);
  bool alt = false;
  cudaError_t e;
  if (sort_precision)
    e = radix_sort_pairs<U128>(c, (U128*)keys, vals, n, true, (U128*)keys_alt, vals_alt, rs, &alt);
  else
    e = radix_sort_pairs<unsigned long long>(c, (unsigned long long*)keys, vals, n, true,
                                             (unsigned long long*)keys_alt, vals_alt, rs, &alt);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return OBVHS_ERR_CUDA;
  }
  launch_k(k_order_out, g, 256, 0, c.stream, alt ? vals_alt : vals, n, order);
  if (cudaGetLastError() != cudaSuccess) return OBVHS_ERR_CUDA;
  uint32_t st = 0;
  if (cudaMemcpyAsync(&st, c.d_status, 4, cudaMemcpyDeviceToHost, c.stream) != cudaSuccess ||
      cudaStreamSynchronize(c.stream) != cudaSuccess) {
    cudaGetLastError();
    return OBVHS_ERR_CUDA;
  }
  if (st & ST_BAD_INPUT) return OBVHS_ERR_BAD_INPUT;
  if (st & (ST_STACK_OVERFLOW | ST_ITER_LIMIT)) return OBVHS_ERR_LIMIT;
  if (st) return OBVHS_ERR_DEVICE;
  return OBVHS_OK;
}

}  // extern "C"
