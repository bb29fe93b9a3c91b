// Device-wide exclusive prefix sum used to turn per-item counts into offsets.
#pragma once

#include "common.cuh"

namespace kups {

constexpr int kScanBlock = 1024;

template <typename T>
__global__ void scan_blocks_kernel(T *data, int64_t n, T *block_sums) {
  __shared__ T scratch[32];
  const int64_t i = (int64_t)blockIdx.x * kScanBlock + threadIdx.x;
  const T v = i < n ? data[i] : T(0);
  T total;
  const T ex = block_exclusive_scan<T>(v, scratch, &total);
  if (i < n) data[i] = ex;
  if (threadIdx.x == 0) block_sums[blockIdx.x] = total;
}

// One block scans the per-block totals sequentially in chunks and writes the
// grand total (if `total` is not null).
template <typename T>
__global__ void scan_sums_kernel(T *block_sums, int64_t nb, T *total) {
  __shared__ T scratch[32];
  T carry = 0;
  for (int64_t base = 0; base < nb; base += kScanBlock) {
    const int64_t i = base + threadIdx.x;
    const T v = i < nb ? block_sums[i] : T(0);
    T chunk;
    const T ex = block_exclusive_scan<T>(v, scratch, &chunk);
    if (i < nb) block_sums[i] = ex + carry;
    carry += chunk;
    __syncthreads();
  }
  if (threadIdx.x == 0 && total != nullptr) *total = carry;
}

template <typename T>
__global__ void scan_add_kernel(T *data, int64_t n, const T *block_sums) {
  const int64_t i = (int64_t)blockIdx.x * kScanBlock + threadIdx.x;
  if (i < n) data[i] += block_sums[blockIdx.x];
}

inline int64_t scan_blocks_needed(int64_t n) { return (n + kScanBlock - 1) / kScanBlock + 1; }

// In-place exclusive scan of data[0..n); `block_sums` has scan_blocks_needed(n)
// entries; `total` (device, may be null) receives the sum of all entries.
template <typename T>
inline cudaError_t exclusive_scan(T *data, int64_t n, T *block_sums, T *total, cudaStream_t s) {
  const int64_t nb = (n + kScanBlock - 1) / kScanBlock;
  if (nb > 0) scan_blocks_kernel<T><<<(unsigned)nb, kScanBlock, 0, s>>>(data, n, block_sums);
  scan_sums_kernel<T><<<1, kScanBlock, 0, s>>>(block_sums, nb, total);
  if (nb > 0) scan_add_kernel<T><<<(unsigned)nb, kScanBlock, 0, s>>>(data, n, block_sums);
  return cudaGetLastError();
}

}  // namespace kups
