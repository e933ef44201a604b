// Synthetic database rows for benchmarks and tests: 256-bit rows with exactly 128 set
// bits, each a pure function of (seed, row number). Not part of the hashing or matching
// path. The construction draws a uniform random 256-bit vector, then clears (or sets)
// uniformly chosen set (or clear) bits until 128 remain. The draw is symmetric under any
// permutation of bit positions, so every 128-subset is equally likely.
#include "ypdq_internal.cuh"

namespace ypdq {

__host__ __device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

__global__ void synth_rows_kernel(uint4* rows, uint64_t n, uint64_t first, uint64_t seed) {
  const uint64_t r = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (r >= n) return;
  uint64_t state = mix64(seed ^ mix64(first + r + 0x9E3779B97F4A7C15ull));
  auto next = [&]() {
    state += 0x9E3779B97F4A7C15ull;
    return mix64(state);
  };
  uint64_t w[4] = {next(), next(), next(), next()};
  int pc = __popcll(w[0]) + __popcll(w[1]) + __popcll(w[2]) + __popcll(w[3]);
  while (pc != 128) {
    const uint32_t pos = static_cast<uint32_t>(next() & 255u);
    const uint64_t bit = 1ull << (pos & 63);
    uint64_t& word = w[pos >> 6];
    if (pc > 128 && (word & bit)) {
      word &= ~bit;
      --pc;
    } else if (pc < 128 && !(word & bit)) {
      word |= bit;
      ++pc;
    }
  }
  rows[2 * r] = make_uint4(static_cast<uint32_t>(w[0]), static_cast<uint32_t>(w[0] >> 32),
                           static_cast<uint32_t>(w[1]), static_cast<uint32_t>(w[1] >> 32));
  rows[2 * r + 1] = make_uint4(static_cast<uint32_t>(w[2]), static_cast<uint32_t>(w[2] >> 32),
                               static_cast<uint32_t>(w[3]), static_cast<uint32_t>(w[3] >> 32));
}

cudaError_t launch_synth_rows(uint8_t* rows, uint64_t n, uint64_t first, uint64_t seed,
                              cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  const unsigned threads = 256;
  const uint64_t blocks = (n + threads - 1) / threads;
  synth_rows_kernel<<<static_cast<unsigned>(blocks), threads, 0, s>>>(
      reinterpret_cast<uint4*>(rows), n, first, seed);
  return cudaGetLastError();
}

}  // namespace ypdq
