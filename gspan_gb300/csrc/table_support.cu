// MNI support of an embedding table that is already in device memory: the
// support step of haozixu/gSpan (support_gpu + support_kernel_v2,
// gspan.cu:165-190, 200-289) for a column-oriented table, one int32 column of
// vertex ids per pattern vertex.  A column's domain is the set of distinct ids
// in it; the support is the smallest non-empty domain (gspan.cu:282-287).
#include "miner.h"

#include <algorithm>

namespace gs {
namespace {

struct TableCols {
    const int32_t* col[kMaxV];
};

__device__ __forceinline__ void table_bit_insert(uint32_t* words, uint32_t v)
{
    uint32_t* w = words + (v >> 5);
    const uint32_t bit = 1u << (v & 31u);
    if (!(__ldcg(w) & bit)) atomicOr(w, bit);
}

// Thread per row: every column's id goes into that column's bitmap.
__global__ void k_table_fill(TableCols t, int32_t ncols, int64_t nrows, int32_t n, uint32_t words,
                             uint32_t* __restrict__ bits, uint32_t* status)
{
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < nrows; r += (int64_t)gridDim.x * blockDim.x) {
        for (int c = 0; c < ncols; ++c) {
            const int32_t v = __ldcs(t.col[c] + r);
            if (v < 0 || v >= n) {
                atomicOr(status, kErrBadGraph);
                continue;
            }
            table_bit_insert(bits + (int64_t)c * words, (uint32_t)v);
        }
    }
}

// Block per column: popcount of its bitmap into out[c].
__global__ void k_table_sizes(uint32_t words, const uint32_t* __restrict__ bits, uint32_t* __restrict__ out)
{
    const uint32_t* b = bits + (int64_t)blockIdx.x * words;
    uint32_t c = 0;
    for (uint32_t i = threadIdx.x; i < words; i += blockDim.x) c += __popc(b[i]);
    for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xFFFFFFFFu, c, o);
    __shared__ uint32_t part[32];
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x < 32) {
        c = threadIdx.x < (blockDim.x >> 5) ? part[threadIdx.x] : 0;
        for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xFFFFFFFFu, c, o);
        if (threadIdx.x == 0) out[blockIdx.x] = c;
    }
}

// out[ncols] = smallest non-zero out[c], or 0x7fffffff when every domain is empty.
__global__ void k_table_min(int32_t ncols, uint32_t* out)
{
    uint32_t best = 0x7fffffffu;
    for (int c = 0; c < ncols; ++c)
        if (out[c] > 0 && out[c] < best) best = out[c];
    out[ncols] = best;
}

cudaError_t launch_table(const TableCols& t, int32_t ncols, int64_t nrows, int32_t n, uint32_t* bits,
                         uint32_t* out, uint32_t* status, cudaStream_t st)
{
    const uint32_t words = (uint32_t)(((int64_t)n + 31) / 32);
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (nrows > 0) {
        const int64_t want = (nrows + 255) / 256;
        const int grid = (int)std::min<int64_t>(want, (int64_t)sms * 8);
        k_table_fill<<<grid, 256, 0, st>>>(t, ncols, nrows, n, words, bits, status);
    }
    k_table_sizes<<<ncols, 256, 0, st>>>(words, bits, out);
    k_table_min<<<1, 1, 0, st>>>(ncols, out);
    return cudaGetLastError();
}

gspan_status check_table_args(int32_t nr_nodes, const int32_t* const* cols, int32_t ncols, int64_t nrows,
                              const uint32_t* out, TableCols* t)
{
    if (!cols || !out || ncols < 1 || ncols > kMaxV || nrows < 0 || nr_nodes < 1) return GSPAN_ERR_INVALID;
    for (int32_t c = 0; c < ncols; ++c) {
        if (!cols[c] && nrows > 0) return GSPAN_ERR_INVALID;
        t->col[c] = cols[c];
    }
    return GSPAN_OK;
}

}  // namespace
}  // namespace gs

extern "C" gspan_status gspan_table_support(gspan_ctx* ctx, int32_t nr_nodes, const int32_t* const* cols,
                                            int32_t ncols, int64_t nrows, uint32_t* out)
{
    if (!ctx) return GSPAN_ERR_INVALID;
    gs::TableCols t{};
    if (gs::check_table_args(nr_nodes, cols, ncols, nrows, out, &t) != GSPAN_OK)
        return gs::fail(ctx, GSPAN_ERR_INVALID, "table support: bad arguments (1..16 columns, nr_nodes >= 1)");
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return gs::cuda_fail(ctx, e, "set device");
    cudaStream_t s = ctx->stream;
    const size_t words = ((size_t)nr_nodes + 31) / 32;
    uint32_t* bits = nullptr;
    uint32_t status = 0;
    if ((e = cudaMallocAsync(&bits, words * ncols * 4, s)) != cudaSuccess) return gs::cuda_fail(ctx, e, "alloc domains");
    if ((e = cudaMemsetAsync(bits, 0, words * ncols * 4, s)) == cudaSuccess &&
        (e = cudaMemsetAsync(ctx->d_status, 0, 4, s)) == cudaSuccess &&
        (e = gs::launch_table(t, ncols, nrows, nr_nodes, bits, out, ctx->d_status, s)) == cudaSuccess)
        e = cudaMemcpyAsync(&status, ctx->d_status, 4, cudaMemcpyDeviceToHost, s);
    cudaFreeAsync(bits, s);
    const cudaError_t e2 = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return gs::cuda_fail(ctx, e, "table support");
    if (e2 != cudaSuccess) return gs::cuda_fail(ctx, e2, "table support");
    if (status) return gs::fail(ctx, GSPAN_ERR_INVALID, "table support: a vertex id is outside [0, nr_nodes)");
    return GSPAN_OK;
}
