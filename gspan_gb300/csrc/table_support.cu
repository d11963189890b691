// MNI support of an embedding table that is already in device memory: the
// support step of haozixu/gSpan (support_gpu + support_kernel_v2,
// gspan.cu:165-190, 200-289) for a column-oriented table, one int32 column of
// vertex ids per pattern vertex.  A column's domain is the set of distinct ids
// in it; the support is the smallest non-empty domain (gspan.cu:282-287).
#include "miner.h"

#include <algorithm>
#include <mutex>

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

// The error of launches just made, cleared once taken.  Callers check with
// cudaPeekAtLastError before launching that no error of earlier, unrelated work
// is pending, so an error seen here is this call's own.
cudaError_t take_launch_error()
{
    const cudaError_t e = cudaPeekAtLastError();
    if (e != cudaSuccess) cudaGetLastError();
    return e;
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
    return take_launch_error();
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
    if ((e = cudaPeekAtLastError()) != cudaSuccess)   // left pending by earlier work: not ours to clear
        return gs::cuda_fail(ctx, e, "table support: an earlier CUDA error is pending on this thread");
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

// ---------------------------------------------------------------------------
// Allocation-free variant of gspan_table_support.
//
// Some callers cannot let this library allocate device memory: a serving
// process that reserved its whole device-memory budget at start-up and must
// not grow or fragment it later, a latency-critical loop that cannot afford
// the device-wide synchronisation cudaMalloc/cudaFree may cause, or a host
// application whose own allocator owns every byte of device memory.  For
// them the domain bitmaps live in a fixed array that is part of this
// library's device image, so the call itself allocates nothing.
//
// The array is 8 MiB on every GPU that loads the library, held until the
// process exits.  Its first 64 words are a header (word 0: bad-id flag); the
// bitmaps follow, so ncols * ceil(nr_nodes / 32) may be at most
// kNoAllocBitmapWords (2,097,088 words: e.g. 16 columns of 4.19M vertices).
// Every call uses the same array and leaves its bitmaps behind; each call
// clears the part it uses before filling it.  Calls whose work overlaps on
// the GPU (another stream, another host thread) race on the array.
//
// The call launches its kernels and returns without waiting.  If an error of
// earlier work is already pending on the calling thread (cudaPeekAtLastError),
// it launches nothing, leaves that error for its owner and returns
// GSPAN_ERR_CUDA; otherwise GSPAN_ERR_CUDA means one of its own launches failed.

namespace gs {
namespace {

constexpr size_t kNoAllocScratchWords = (size_t)2 << 20;   // 8 MiB
constexpr size_t kNoAllocHeaderWords = 64;                 // 256 bytes
constexpr size_t kNoAllocBitmapWords = kNoAllocScratchWords - kNoAllocHeaderWords;
constexpr int kNoAllocMaxDevices = 64;

static __device__ __align__(256) uint32_t g_table_scratch[kNoAllocScratchWords];

std::mutex g_scratch_mu;
uint32_t* g_scratch_addr[kNoAllocMaxDevices] = {};

// Device address of g_table_scratch on device `dev` (which must be current).
// In host code the symbol is only a host-side stand-in, so the address is
// fetched once per device with cudaGetSymbolAddress and cached.
gspan_status scratch_for(int dev, uint32_t** out)
{
    if (dev < 0 || dev >= kNoAllocMaxDevices) return GSPAN_ERR_LIMIT;
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_table_scratch);
        if (e != cudaSuccess || !p) return GSPAN_ERR_CUDA;
        g_scratch_addr[dev] = static_cast<uint32_t*>(p);
    }
    *out = g_scratch_addr[dev];
    return GSPAN_OK;
}

__global__ void k_scratch_clear(uint32_t* __restrict__ words, int64_t count)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x)
        words[i] = 0u;
}

// Like k_table_min, but out[ncols] = 0xFFFFFFFF when the fill saw an id
// outside [0, nr_nodes) (the call is asynchronous and cannot return it).
__global__ void k_table_min_flagged(int32_t ncols, const uint32_t* __restrict__ flag, uint32_t* out)
{
    uint32_t best = 0x7fffffffu;
    for (int c = 0; c < ncols; ++c)
        if (out[c] > 0 && out[c] < best) best = out[c];
    out[ncols] = *flag ? 0xFFFFFFFFu : best;
}

}  // namespace
}  // namespace gs

extern "C" gspan_status gspan_table_support_noalloc(int32_t nr_nodes, const int32_t* const* cols, int32_t ncols,
                                                    int64_t nrows, uint32_t* out, void* stream)
{
    gs::TableCols t{};
    if (gs::check_table_args(nr_nodes, cols, ncols, nrows, out, &t) != GSPAN_OK) return GSPAN_ERR_INVALID;
    const size_t words = ((size_t)nr_nodes + 31) / 32;
    if ((size_t)ncols * words > gs::kNoAllocBitmapWords) return GSPAN_ERR_LIMIT;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return GSPAN_ERR_NO_DEVICE;
    uint32_t* scratch = nullptr;
    const gspan_status rc = gs::scratch_for(dev, &scratch);
    if (rc != GSPAN_OK) return rc;
    if (cudaPeekAtLastError() != cudaSuccess) return GSPAN_ERR_CUDA;   // earlier work's error, left pending
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    uint32_t* flag = scratch;
    uint32_t* bits = scratch + gs::kNoAllocHeaderWords;
    const int64_t used = (int64_t)gs::kNoAllocHeaderWords + (int64_t)ncols * (int64_t)words;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int grid = (int)std::min<int64_t>((used + 255) / 256, (int64_t)(sms > 0 ? sms : 1) * 8);
    gs::k_scratch_clear<<<grid, 256, 0, s>>>(scratch, used);
    if (nrows > 0) {
        const int fgrid = (int)std::min<int64_t>((nrows + 255) / 256, (int64_t)(sms > 0 ? sms : 1) * 8);
        gs::k_table_fill<<<fgrid, 256, 0, s>>>(t, ncols, nrows, nr_nodes, (uint32_t)words, bits, flag);
    }
    gs::k_table_sizes<<<ncols, 256, 0, s>>>((uint32_t)words, bits, out);
    gs::k_table_min_flagged<<<1, 1, 0, s>>>(ncols, flag, out);
    return gs::take_launch_error() == cudaSuccess ? GSPAN_OK : GSPAN_ERR_CUDA;
}
