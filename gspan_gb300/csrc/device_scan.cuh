// Device scans shared by the device-side graph builders (the text loader and
// the label-frequency pruning): a 256-thread block scan, a one-block scan of
// block sums, and the two passes of a dense ranking of byte flags.
#pragma once

#include <cstdint>

namespace gs {
namespace {

constexpr unsigned kAll = 0xFFFFFFFFu;
constexpr int kThreads = 256;
constexpr int kPer = 8;                      // elements per thread in the scans
constexpr int kChunk = kThreads * kPer;      // elements per scan block

// Exclusive scan of one value per thread over a 256-thread block; *total
// receives the block's sum.
__device__ int64_t block_exclusive_scan(int64_t v, int64_t* total)
{
    __shared__ int64_t warp_sums[kThreads / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int64_t x = v;
    for (int d = 1; d < 32; d <<= 1) {
        const int64_t y = __shfl_up_sync(kAll, x, d);
        if (lane >= d) x += y;
    }
    if (lane == 31) warp_sums[w] = x;
    __syncthreads();
    if (w == 0) {
        int64_t s = lane < kThreads / 32 ? warp_sums[lane] : 0;
        for (int d = 1; d < 32; d <<= 1) {
            const int64_t y = __shfl_up_sync(kAll, s, d);
            if (lane >= d) s += y;
        }
        if (lane < kThreads / 32) warp_sums[lane] = s;
    }
    __syncthreads();
    const int64_t base = w > 0 ? warp_sums[w - 1] : 0;
    *total = warp_sums[kThreads / 32 - 1];
    __syncthreads();
    return base + x - v;
}

// Exclusive scan of n int64 values in one block of 1024 threads (block sums
// of the other scans: a few hundred thousand at most); out[n] = total.
__global__ void k_scan_small(const int64_t* __restrict__ in, int64_t* __restrict__ out, int64_t n)
{
    __shared__ int64_t part[1024];
    const int64_t per = (n + blockDim.x - 1) / blockDim.x;
    const int64_t b = (int64_t)threadIdx.x * per, e = b + per < n ? b + per : n;
    int64_t s = 0;
    for (int64_t i = b; i < e; ++i) s += in[i];
    part[threadIdx.x] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        int64_t run = 0;
        for (unsigned t = 0; t < blockDim.x; ++t) {
            const int64_t v = part[t];
            part[t] = run;
            run += v;
        }
        out[n] = run;
    }
    __syncthreads();
    int64_t run = part[threadIdx.x];
    for (int64_t i = b; i < e; ++i) {
        const int64_t v = in[i];
        out[i] = run;
        run += v;
    }
}

// Exclusive scan of byte flags in blocks of kChunk: pass 1 block sums.
__global__ void k_flag_count(const uint8_t* __restrict__ flag, int64_t n, int64_t* __restrict__ block_count)
{
    const int64_t i0 = (int64_t)blockIdx.x * kChunk + (int64_t)threadIdx.x * kPer;
    int64_t c = 0;
    for (int q = 0; q < kPer; ++q)
        if (i0 + q < n) c += flag[i0 + q];
    int64_t total;
    block_exclusive_scan(c, &total);
    if (threadIdx.x == 0) block_count[blockIdx.x] = total;
}

// Pass 2: dense rank of every present id.
__global__ void k_flag_rank(const uint8_t* __restrict__ flag, int64_t n, const int64_t* __restrict__ block_off,
                            int32_t* __restrict__ rank)
{
    const int64_t i0 = (int64_t)blockIdx.x * kChunk + (int64_t)threadIdx.x * kPer;
    int64_t c = 0;
    for (int q = 0; q < kPer; ++q)
        if (i0 + q < n) c += flag[i0 + q];
    int64_t total;
    int64_t at = block_off[blockIdx.x] + block_exclusive_scan(c, &total);
    for (int q = 0; q < kPer; ++q)
        if (i0 + q < n) {
            rank[i0 + q] = flag[i0 + q] ? (int32_t)at : -1;
            at += flag[i0 + q];
        }
}

}  // namespace
}  // namespace gs
