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

// Row `row` of the 128-bit generator for `seed`.
__device__ __forceinline__ void synth_row(uint64_t seed, uint64_t row, uint64_t w[4]) {
  uint64_t state = mix64(seed ^ mix64(row + 0x9E3779B97F4A7C15ull));
  auto next = [&]() {
    state += 0x9E3779B97F4A7C15ull;
    return mix64(state);
  };
  w[0] = next();
  w[1] = next();
  w[2] = next();
  w[3] = next();
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
}

__device__ __forceinline__ void store_row(uint4* rows, uint64_t r, const uint64_t w[4]) {
  rows[2 * r] = make_uint4(static_cast<uint32_t>(w[0]), static_cast<uint32_t>(w[0] >> 32),
                           static_cast<uint32_t>(w[1]), static_cast<uint32_t>(w[1] >> 32));
  rows[2 * r + 1] = make_uint4(static_cast<uint32_t>(w[2]), static_cast<uint32_t>(w[2] >> 32),
                               static_cast<uint32_t>(w[3]), static_cast<uint32_t>(w[3] >> 32));
}

__global__ void synth_rows_kernel(uint4* rows, uint64_t n, uint64_t first, uint64_t seed) {
  const uint64_t r = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (r >= n) return;
  uint64_t w[4];
  synth_row(seed, first + r, w);
  store_row(rows, r, w);
}

// Clustered rows: global row g belongs to centre c = g / members, the 128-bit generator's
// row c for `seed`; the member flips d distinct bits of it, d = popcount of `trials` random
// bits (Binomial(trials, 1/2)), positions drawn from a second per-row stream.
__global__ void synth_clustered_kernel(uint4* rows, uint64_t n, uint64_t first, uint64_t members,
                                       uint32_t trials, uint64_t seed) {
  const uint64_t r = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (r >= n) return;
  const uint64_t g = first + r;
  uint64_t w[4];
  synth_row(seed, g / members, w);
  uint64_t state = mix64((seed ^ 0xC13FA9A902A6328Full) ^ mix64(g + 0x632BE59BD9B4E019ull));
  auto next = [&]() {
    state += 0x9E3779B97F4A7C15ull;
    return mix64(state);
  };
  const uint64_t mask = trials >= 64 ? ~0ull : ((1ull << trials) - 1);
  const int d = __popcll(next() & mask);
  uint64_t f[4] = {0, 0, 0, 0};
  for (int k = 0; k < d;) {
    const uint32_t pos = static_cast<uint32_t>(next() & 255u);
    const uint64_t bit = 1ull << (pos & 63);
    if (!(f[pos >> 6] & bit)) {
      f[pos >> 6] |= bit;
      ++k;
    }
  }
  for (int k = 0; k < 4; ++k) w[k] ^= f[k];
  store_row(rows, r, w);
}

cudaError_t launch_synth_clustered(uint8_t* rows, uint64_t n, uint64_t first, uint64_t members,
                                   uint32_t trials, uint64_t seed, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  const unsigned threads = 256;
  const uint64_t blocks = (n + threads - 1) / threads;
  synth_clustered_kernel<<<static_cast<unsigned>(blocks), threads, 0, s>>>(
      reinterpret_cast<uint4*>(rows), n, first, members, trials, seed);
  return cudaGetLastError();
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
