// Stable LSD radix sort of (uint32 key, uint32 value) pairs on the device.
//
// Used to order cells by cell-list bin.  Each pass sorts on one 8-bit digit:
//   1. count:   per tile of kTile elements, a histogram of the digit
//               (stored digit-major: counts[digit * ntiles + tile]);
//   2. scan:    one block forms the exclusive prefix sum of all counts, which
//               is the output offset of each (digit, tile) run;
//   3. scatter: per tile, each element's rank among equal digits of lower
//               index in the tile (warp match + per-warp counts), added to
//               its run's offset.
// Elements with equal keys keep their input order, so the result is the
// same as any stable host sort of the same pairs.
#include "radix_sort.cuh"

namespace dpm {

namespace {

constexpr int kThreads = 256;
constexpr int kRounds = 4;
constexpr int kTile = kThreads * kRounds;
constexpr int kDigits = 256;
constexpr int kWarps = kThreads / 32;

__global__ void __launch_bounds__(kThreads)
    radix_count(const uint32_t *__restrict__ keys, int n, int shift,
                uint32_t *__restrict__ counts, int ntiles) {
  __shared__ uint32_t hist[kDigits];
  for (int d = threadIdx.x; d < kDigits; d += kThreads) hist[d] = 0;
  __syncthreads();
  const int base = blockIdx.x * kTile;
#pragma unroll
  for (int r = 0; r < kRounds; ++r) {
    int i = base + r * kThreads + threadIdx.x;
    if (i < n) atomicAdd(&hist[(keys[i] >> shift) & 0xffu], 1u);
  }
  __syncthreads();
  for (int d = threadIdx.x; d < kDigits; d += kThreads)
    counts[(size_t)d * ntiles + blockIdx.x] = hist[d];
}

// Exclusive scan of m counters by one block of 1024 threads.
__global__ void __launch_bounds__(1024)
    radix_scan(uint32_t *__restrict__ counts, int m) {
  __shared__ uint32_t part[1024];
  const int t = threadIdx.x;
  const int chunk = (m + 1023) / 1024;
  const int b = t * chunk, e = min(m, b + chunk);
  uint32_t s = 0;
  for (int i = b; i < e; ++i) s += counts[i];
  part[t] = s;
  __syncthreads();
  // Hillis-Steele inclusive scan over the 1024 partial sums.
  for (int o = 1; o < 1024; o <<= 1) {
    uint32_t v = t >= o ? part[t - o] : 0u;
    __syncthreads();
    part[t] += v;
    __syncthreads();
  }
  uint32_t run = part[t] - s;
  for (int i = b; i < e; ++i) {
    uint32_t c = counts[i];
    counts[i] = run;
    run += c;
  }
}

__global__ void __launch_bounds__(kThreads)
    radix_scatter(const uint32_t *__restrict__ kin, const uint32_t *__restrict__ vin,
                  uint32_t *__restrict__ kout, uint32_t *__restrict__ vout, int n,
                  int shift, const uint32_t *__restrict__ offsets, int ntiles) {
  __shared__ uint32_t base[kDigits];
  __shared__ uint32_t running[kDigits];
  __shared__ uint16_t wcount[kWarps][kDigits];
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  for (int d = t; d < kDigits; d += kThreads) {
    base[d] = offsets[(size_t)d * ntiles + blockIdx.x];
    running[d] = 0;
  }
  for (int i = t; i < kWarps * kDigits; i += kThreads) (&wcount[0][0])[i] = 0;
  __syncthreads();
  const unsigned lt_mask = (1u << lane) - 1u;
  for (int r = 0; r < kRounds; ++r) {
    const int i = blockIdx.x * kTile + r * kThreads + t;
    const bool valid = i < n;
    uint32_t key = valid ? kin[i] : 0u;
    uint32_t val = valid ? vin[i] : 0u;
    // invalid elements use digit 256, which matches no valid digit
    const unsigned d = valid ? ((key >> shift) & 0xffu) : 256u;
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    const unsigned rank = __popc(peers & lt_mask);
    if (valid && rank == 0) wcount[w][d] = (uint16_t)__popc(peers);
    __syncthreads();
    if (valid) {
      uint32_t before = 0;
      for (int q = 0; q < w; ++q) before += wcount[q][d];
      const uint32_t dst = base[d] + running[d] + before + rank;
      kout[dst] = key;
      vout[dst] = val;
    }
    __syncthreads();
    for (int dd = t; dd < kDigits; dd += kThreads) {
      uint32_t s = 0;
      for (int q = 0; q < kWarps; ++q) {
        s += wcount[q][dd];
        wcount[q][dd] = 0;
      }
      running[dd] += s;
    }
    __syncthreads();
  }
}

} // namespace

size_t radix_sort_scratch_bytes(int n) {
  const int ntiles = (n + kTile - 1) / kTile;
  return sizeof(uint32_t) * ((size_t)kDigits * ntiles) + 256;
}

int radix_sort_passes(int key_bits) { return (key_bits + 7) / 8; }

cudaError_t radix_sort_pairs(uint32_t *keys, uint32_t *vals, uint32_t *keys_alt,
                             uint32_t *vals_alt, int n, int key_bits,
                             uint32_t *scratch, cudaStream_t stream,
                             bool *result_in_alt) {
  const int ntiles = (n + kTile - 1) / kTile;
  const int passes = radix_sort_passes(key_bits);
  uint32_t *ka = keys, *va = vals, *kb = keys_alt, *vb = vals_alt;
  for (int p = 0; p < passes; ++p) {
    const int shift = 8 * p;
    radix_count<<<ntiles, kThreads, 0, stream>>>(ka, n, shift, scratch, ntiles);
    radix_scan<<<1, 1024, 0, stream>>>(scratch, kDigits * ntiles);
    radix_scatter<<<ntiles, kThreads, 0, stream>>>(ka, va, kb, vb, n, shift, scratch,
                                                   ntiles);
    uint32_t *tk = ka, *tv = va;
    ka = kb;
    va = vb;
    kb = tk;
    vb = tv;
  }
  *result_in_alt = (passes % 2) == 1;
  return cudaGetLastError();
}

} // namespace dpm
