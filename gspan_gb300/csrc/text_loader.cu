// Device-side loader for the gSpan text format (graph.cc:38-64 `from_txt`,
// graph.cc:66-112 the CSR construction, convert.cc:6-16): tokens, records,
// dense vertex numbering and the CSR are built on the GPU from the raw file
// bytes, then the device store exactly as gspan_graph_upload builds it.
//
// Semantics follow the token-driven reader: a token starting with 't' takes
// a string and an integer, 'v' an id and a label, 'e' two ids and a label;
// other tokens are skipped.  Vertices are created by any mention, label 0
// until a 'v' record names one (the last one wins), renumbered densely in
// ascending id order; every edge is entered at both ends.  Whether a token is
// a record head depends on all tokens before it; that is resolved exactly by
// a scan over per-token transition functions of "arguments still owed" (0..3).
//
// Text this token parser would not read exactly like the reference's
// scanf-based reader is refused (GSPAN_ERR_INVALID), never guessed at or cut
// short: a record whose integer fails to parse or that the end of the text
// cuts off (the reference then reuses the previous record's values, which the
// host reader reproduces), an integer followed by other characters in one
// token ("12ab"), an integer outside int32, or a token of 64 characters or
// more.  Everything else gives exactly the host reader's graph.
#include "device_scan.cuh"
#include "miner.h"

#include <cstdint>
#include <vector>

namespace gs {
namespace {

constexpr int kTokPer = 32;                  // tokens per thread in the head scan
constexpr int kLongToken = 64;

enum : uint8_t { kIntOk = 0, kIntFail = 1, kIntBad = 2 };

__device__ __forceinline__ bool is_space(uint8_t c)
{
    return c == ' ' || c == '\t' || c == '\n' || c == '\v' || c == '\f' || c == '\r';
}

// ---- token starts: count per block, scan, write ----------------------------

__device__ __forceinline__ bool token_start(const uint8_t* t, int64_t i)
{
    return !is_space(t[i]) && (i == 0 || is_space(t[i - 1]));
}

__global__ void k_tok_count(const uint8_t* __restrict__ text, int64_t len, int64_t* __restrict__ block_count)
{
    const int64_t i0 = (int64_t)blockIdx.x * kChunk + (int64_t)threadIdx.x * kPer;
    int64_t c = 0;
    for (int q = 0; q < kPer; ++q)
        if (i0 + q < len) c += token_start(text, i0 + q);
    int64_t total;
    block_exclusive_scan(c, &total);
    if (threadIdx.x == 0) block_count[blockIdx.x] = total;
}

__global__ void k_tok_write(const uint8_t* __restrict__ text, int64_t len, const int64_t* __restrict__ block_off,
                            int32_t* __restrict__ tok)
{
    const int64_t i0 = (int64_t)blockIdx.x * kChunk + (int64_t)threadIdx.x * kPer;
    int64_t c = 0;
    for (int q = 0; q < kPer; ++q)
        if (i0 + q < len) c += token_start(text, i0 + q);
    int64_t total;
    int64_t at = block_off[blockIdx.x] + block_exclusive_scan(c, &total);
    for (int q = 0; q < kPer; ++q)
        if (i0 + q < len && token_start(text, i0 + q)) tok[at++] = (int32_t)(i0 + q);
}

// ---- per-token facts ---------------------------------------------------------

// Head class: arguments a record head takes ('t', 'v': 2, 'e': 3, else 0).
__device__ __forceinline__ int head_args(uint8_t c) { return c == 'e' ? 3 : (c == 't' || c == 'v') ? 2 : 0; }

// Transition of "arguments still owed" across one token, 4 entries x 2 bits.
__device__ __forceinline__ uint8_t token_fn(int hc)
{
    // f(0) = hc, f(s) = s - 1 for s = 1..3.
    return (uint8_t)(hc | (0 << 2) | (1 << 4) | (2 << 6));
}
__device__ __forceinline__ int apply_fn(uint8_t f, int s) { return (f >> (2 * s)) & 3; }
// (g after f)
__device__ __forceinline__ uint8_t compose(uint8_t g, uint8_t f)
{
    uint8_t r = 0;
    for (int s = 0; s < 4; ++s) r |= (uint8_t)(apply_fn(g, apply_fn(f, s)) << (2 * s));
    return r;
}
constexpr uint8_t kIdentity = (uint8_t)(0 | (1 << 2) | (2 << 4) | (3 << 6));

__global__ void k_tok_info(const uint8_t* __restrict__ text, int64_t len, const int32_t* __restrict__ tok, int64_t ntok,
                           uint8_t* __restrict__ fn, uint8_t* __restrict__ ist, int32_t* __restrict__ val,
                           uint8_t* __restrict__ islong)
{
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < ntok; j += (int64_t)gridDim.x * blockDim.x) {
        const int64_t p = tok[j];
        int64_t q = p;
        while (q < len && q - p < kLongToken && !is_space(text[q])) ++q;
        islong[j] = q - p >= kLongToken;
        const uint8_t c = text[p];
        fn[j] = token_fn(head_args(c));
        // As an integer: optional sign, digits, nothing else.
        int64_t k = p;
        bool neg = false;
        if (text[k] == '+' || text[k] == '-') {
            neg = text[k] == '-';
            ++k;
        }
        uint8_t st = kIntOk;
        int64_t v = 0;
        if (k >= q || text[k] < '0' || text[k] > '9') {
            st = kIntFail;   // nothing an integer can start with: the reader stops here
        } else {
            for (; k < q && text[k] >= '0' && text[k] <= '9'; ++k) {
                v = v * 10 + (text[k] - '0');
                if (v > 2147483648ll) break;
            }
            const int64_t sv = neg ? -v : v;
            if (k < q || sv > 2147483647ll || sv < -2147483648ll || q - p >= kLongToken) st = kIntBad;
            v = sv;
        }
        ist[j] = st;
        val[j] = st == kIntOk ? (int32_t)v : 0;
    }
}

// ---- record heads: scan of transition functions --------------------------------

__global__ void k_fn_blocks(const uint8_t* __restrict__ fn, int64_t ntok, uint8_t* __restrict__ block_fn)
{
    __shared__ uint8_t tf[kThreads];
    const int64_t j0 = ((int64_t)blockIdx.x * kThreads + threadIdx.x) * kTokPer;
    uint8_t F = kIdentity;
    for (int q = 0; q < kTokPer; ++q)
        if (j0 + q < ntok) F = compose(fn[j0 + q], F);
    tf[threadIdx.x] = F;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint8_t B = kIdentity;
        for (int t = 0; t < kThreads; ++t) B = compose(tf[t], B);
        block_fn[blockIdx.x] = B;
    }
}

__global__ void k_fn_states(const uint8_t* __restrict__ block_fn, int64_t nblocks, uint8_t* __restrict__ block_state)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    int s = 0;
    for (int64_t b = 0; b < nblocks; ++b) {
        block_state[b] = (uint8_t)s;
        s = apply_fn(block_fn[b], s);
    }
}

__global__ void k_heads(const uint8_t* __restrict__ fn, int64_t ntok, const uint8_t* __restrict__ block_state,
                        uint8_t* __restrict__ head)
{
    __shared__ uint8_t tf[kThreads];
    __shared__ uint8_t ts[kThreads];
    const int64_t j0 = ((int64_t)blockIdx.x * kThreads + threadIdx.x) * kTokPer;
    uint8_t F = kIdentity;
    for (int q = 0; q < kTokPer; ++q)
        if (j0 + q < ntok) F = compose(fn[j0 + q], F);
    tf[threadIdx.x] = F;
    __syncthreads();
    if (threadIdx.x == 0) {
        int s = block_state[blockIdx.x];
        for (int t = 0; t < kThreads; ++t) {
            ts[t] = (uint8_t)s;
            s = apply_fn(tf[t], s);
        }
    }
    __syncthreads();
    int s = ts[threadIdx.x];
    for (int q = 0; q < kTokPer; ++q) {
        if (j0 + q >= ntok) break;
        head[j0 + q] = s == 0;
        s = apply_fn(fn[j0 + q], s);
    }
}

// ---- records ---------------------------------------------------------------------

// Earliest record the loader refuses: (head index << 1) | character-level
// (0: a field that is not an integer, or a record cut off by the end).
__global__ void k_records_end(const uint8_t* __restrict__ text, const int32_t* __restrict__ tok, int64_t ntok,
                              const uint8_t* __restrict__ head, const uint8_t* __restrict__ ist,
                              const uint8_t* __restrict__ islong, unsigned long long* __restrict__ end)
{
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < ntok; j += (int64_t)gridDim.x * blockDim.x) {
        if (!head[j]) continue;
        const uint8_t c = text[tok[j]];
        const int na = head_args(c);
        int ev = -1;   // -1 none, 0 stop, 1 unsupported
        if (islong[j]) {
            ev = 1;
        } else if (na > 0) {
            if (j + na >= ntok) {
                ev = 0;   // cut off by the end of the text
            } else if (c == 't') {
                if (islong[j + 1]) ev = 1;
                else if (ist[j + 2] == kIntBad) ev = 1;
                else if (ist[j + 2] == kIntFail) ev = 0;
            } else {
                for (int a = 1; a <= na && ev < 0; ++a) {
                    if (ist[j + a] == kIntBad) ev = 1;
                    else if (ist[j + a] == kIntFail) ev = 0;
                }
            }
        }
        if (ev >= 0) atomicMin(end, ((unsigned long long)j << 1) | (unsigned long long)ev);
    }
}

// Valid 'v' and 'e' records before the end: appended (order kept for 'v').
__global__ void k_records(const uint8_t* __restrict__ text, const int32_t* __restrict__ tok, int64_t ntok,
                          const uint8_t* __restrict__ head, const int32_t* __restrict__ val, int64_t stop,
                          int4* __restrict__ vrec, int4* __restrict__ erec, unsigned long long* __restrict__ counts,
                          int32_t* __restrict__ idminmax)
{
    const int lane = threadIdx.x & 31;
    int32_t lo = INT32_MAX, hi = INT32_MIN;
    for (int64_t base = blockIdx.x * (int64_t)blockDim.x; base < ntok; base += (int64_t)gridDim.x * blockDim.x) {
        const int64_t j = base + threadIdx.x;
        const bool ok = j < ntok && j < stop && head[j];
        const uint8_t c = ok ? text[tok[j]] : 0;
        const bool isv = c == 'v', ise = c == 'e';
        const unsigned vm = __ballot_sync(kAll, isv), em = __ballot_sync(kAll, ise);
        unsigned long long vb = 0, eb = 0;
        if (lane == 0 && vm) vb = atomicAdd(counts + 0, (unsigned long long)__popc(vm));
        if (lane == 0 && em) eb = atomicAdd(counts + 1, (unsigned long long)__popc(em));
        vb = __shfl_sync(kAll, vb, 0);
        eb = __shfl_sync(kAll, eb, 0);
        const unsigned below = (1u << lane) - 1u;
        if (isv) {
            const int32_t id = val[j + 1];
            vrec[vb + __popc(vm & below)] = make_int4(id, val[j + 2], (int32_t)j, 0);
            lo = min(lo, id);
            hi = max(hi, id);
        }
        if (ise) {
            const int32_t u = val[j + 1], v = val[j + 2];
            erec[eb + __popc(em & below)] = make_int4(u, v, val[j + 3], 0);
            lo = min(lo, min(u, v));
            hi = max(hi, max(u, v));
        }
    }
    for (int d = 16; d > 0; d >>= 1) {
        lo = min(lo, __shfl_xor_sync(kAll, lo, d));
        hi = max(hi, __shfl_xor_sync(kAll, hi, d));
    }
    if (lane == 0) {
        atomicMin(idminmax + 0, lo);
        atomicMax(idminmax + 1, hi);
    }
}

// ---- vertices and edges ----------------------------------------------------------

__global__ void k_id_flags(const int4* __restrict__ vrec, int64_t nv, const int4* __restrict__ erec, int64_t ne,
                           int32_t idlo, uint8_t* __restrict__ flag)
{
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nv; i += stride)
        flag[(int64_t)vrec[i].x - idlo] = 1;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < ne; i += stride) {
        flag[(int64_t)erec[i].x - idlo] = 1;
        flag[(int64_t)erec[i].y - idlo] = 1;
    }
}

__global__ void k_vertex_labels(const int4* __restrict__ vrec, int64_t nv, int32_t idlo, const int32_t* __restrict__ rank,
                                int32_t* __restrict__ last, int pass, int32_t* __restrict__ vlabel)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nv; i += (int64_t)gridDim.x * blockDim.x) {
        const int4 r = vrec[i];
        const int32_t d = rank[(int64_t)r.x - idlo];
        if (pass == 0)
            atomicMax(last + d, r.z);      // the last 'v' record of a vertex names its label
        else if (last[d] == r.z)
            vlabel[d] = r.y;
    }
}

__global__ void k_degrees(const int4* __restrict__ erec, int64_t ne, int32_t idlo, const int32_t* __restrict__ rank,
                          int64_t* __restrict__ deg)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < ne; i += (int64_t)gridDim.x * blockDim.x) {
        const int4 r = erec[i];
        atomicAdd((unsigned long long*)(deg + rank[(int64_t)r.x - idlo]), 1ull);
        atomicAdd((unsigned long long*)(deg + rank[(int64_t)r.y - idlo]), 1ull);
    }
}

__global__ void k_offsets32(const int64_t* __restrict__ off64, int64_t n1, int32_t* __restrict__ off,
                            unsigned long long* __restrict__ cursor)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n1; i += (int64_t)gridDim.x * blockDim.x) {
        off[i] = (int32_t)off64[i];
        cursor[i] = (unsigned long long)off64[i];
    }
}

__global__ void k_scatter_edges(const int4* __restrict__ erec, int64_t ne, int32_t idlo, const int32_t* __restrict__ rank,
                                unsigned long long* __restrict__ cursor, gspan_edge* __restrict__ edges)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < ne; i += (int64_t)gridDim.x * blockDim.x) {
        const int4 r = erec[i];
        const int32_t du = rank[(int64_t)r.x - idlo], dv = rank[(int64_t)r.y - idlo];
        const unsigned long long p = atomicAdd(cursor + du, 1ull);
        edges[p] = gspan_edge{du, dv, r.z};
        const unsigned long long q = atomicAdd(cursor + dv, 1ull);
        edges[q] = gspan_edge{dv, du, r.z};
    }
}

int grid_of(int64_t work)
{
    const int64_t b = (work + kThreads - 1) / kThreads;
    return (int)(b < 1 ? 1 : (b > 4096 ? 4096 : b));
}

}  // namespace

gspan_status load_text(gspan_ctx* ctx, const char* text, int64_t len, gspan_graph** out, int32_t* nr_nodes,
                       int32_t* nr_edges)
{
    if (len < 0 || len >= ((int64_t)1 << 31) - 1 || (len > 0 && !text))
        return fail(ctx, GSPAN_ERR_INVALID, "text must be below 2^31 bytes");
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "set device");
    cudaStream_t s = ctx->stream;
    std::vector<void*> tmp;
    auto freeall = [&]() {
        for (void* p : tmp) cudaFreeAsync(p, s);
        cudaStreamSynchronize(s);
        tmp.clear();
    };
    auto alloc = [&](void** p, size_t bytes) {
        *p = nullptr;
        const cudaError_t r = cudaMallocAsync(p, bytes < 16 ? 16 : bytes, s);
        if (r == cudaSuccess) tmp.push_back(*p);
        return r;
    };
#define LT_CK(call, what)                      \
    do {                                       \
        if ((e = (call)) != cudaSuccess) {     \
            freeall();                         \
            return cuda_fail(ctx, e, what);    \
        }                                      \
    } while (0)
    auto read = [&](void* dst, const void* src, size_t bytes) {
        cudaError_t r = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, s);
        if (r == cudaSuccess) r = cudaStreamSynchronize(s);
        return r;
    };

    // Tokens.
    uint8_t* d_text = nullptr;
    LT_CK(alloc((void**)&d_text, (size_t)len), "alloc text");
    if (len > 0) LT_CK(cudaMemcpyAsync(d_text, text, (size_t)len, cudaMemcpyHostToDevice, s), "copy text");
    const int64_t nb = (len + kChunk - 1) / kChunk;
    int64_t *d_bc = nullptr, *d_bo = nullptr;
    LT_CK(alloc((void**)&d_bc, (size_t)(nb + 1) * 8), "alloc block counts");
    LT_CK(alloc((void**)&d_bo, (size_t)(nb + 1) * 8), "alloc block offsets");
    int64_t ntok = 0;
    if (nb > 0) {
        k_tok_count<<<(int)nb, kThreads, 0, s>>>(d_text, len, d_bc);
        k_scan_small<<<1, 1024, 0, s>>>(d_bc, d_bo, nb);
        LT_CK(cudaGetLastError(), "token count launch");
        LT_CK(read(&ntok, d_bo + nb, 8), "token count");
    }
    int32_t* d_tok = nullptr;
    uint8_t *d_fn = nullptr, *d_ist = nullptr, *d_long = nullptr, *d_head = nullptr;
    int32_t* d_val = nullptr;
    LT_CK(alloc((void**)&d_tok, (size_t)ntok * 4), "alloc tokens");
    LT_CK(alloc((void**)&d_fn, (size_t)ntok), "alloc tokens");
    LT_CK(alloc((void**)&d_ist, (size_t)ntok), "alloc tokens");
    LT_CK(alloc((void**)&d_long, (size_t)ntok), "alloc tokens");
    LT_CK(alloc((void**)&d_head, (size_t)ntok), "alloc tokens");
    LT_CK(alloc((void**)&d_val, (size_t)ntok * 4), "alloc tokens");
    unsigned long long end = ~0ull;
    unsigned long long* d_end = nullptr;
    unsigned long long* d_cnt = nullptr;
    int32_t* d_mm = nullptr;
    LT_CK(alloc((void**)&d_end, 8), "alloc scalars");
    LT_CK(alloc((void**)&d_cnt, 16), "alloc scalars");
    LT_CK(alloc((void**)&d_mm, 8), "alloc scalars");
    const int32_t mm0[2] = {INT32_MAX, INT32_MIN};
    LT_CK(cudaMemcpyAsync(d_end, &end, 8, cudaMemcpyHostToDevice, s), "init scalars");
    LT_CK(cudaMemsetAsync(d_cnt, 0, 16, s), "init scalars");
    LT_CK(cudaMemcpyAsync(d_mm, mm0, 8, cudaMemcpyHostToDevice, s), "init scalars");
    int4 *d_vrec = nullptr, *d_erec = nullptr;
    LT_CK(alloc((void**)&d_vrec, (size_t)(ntok / 3 + 1) * sizeof(int4)), "alloc records");
    LT_CK(alloc((void**)&d_erec, (size_t)(ntok / 4 + 1) * sizeof(int4)), "alloc records");
    unsigned long long cnt[2] = {0, 0};
    if (ntok > 0) {
        k_tok_write<<<(int)nb, kThreads, 0, s>>>(d_text, len, d_bo, d_tok);
        k_tok_info<<<grid_of(ntok), kThreads, 0, s>>>(d_text, len, d_tok, ntok, d_fn, d_ist, d_val, d_long);
        const int64_t hb = (ntok + (int64_t)kThreads * kTokPer - 1) / ((int64_t)kThreads * kTokPer);
        uint8_t *d_bfn = nullptr, *d_bst = nullptr;
        LT_CK(alloc((void**)&d_bfn, (size_t)hb), "alloc head scan");
        LT_CK(alloc((void**)&d_bst, (size_t)hb), "alloc head scan");
        k_fn_blocks<<<(int)hb, kThreads, 0, s>>>(d_fn, ntok, d_bfn);
        k_fn_states<<<1, 32, 0, s>>>(d_bfn, hb, d_bst);
        k_heads<<<(int)hb, kThreads, 0, s>>>(d_fn, ntok, d_bst, d_head);
        k_records_end<<<grid_of(ntok), kThreads, 0, s>>>(d_text, d_tok, ntok, d_head, d_ist, d_long, d_end);
        LT_CK(cudaGetLastError(), "token launches");
        LT_CK(read(&end, d_end, 8), "record end");
        if (end != ~0ull && (end & 1)) {
            freeall();
            return fail(ctx, GSPAN_ERR_INVALID,
                        "text has a token the device loader does not read like the reference's scanf-based reader "
                        "(an integer followed by other characters, an integer outside int32, or a token of 64 "
                        "characters or more); load it with the host reader");
        }
        if (end != ~0ull) {
            freeall();
            return fail(ctx, GSPAN_ERR_INVALID,
                        "text has a record with a field that is not an integer, or cut off by the end of the text; "
                        "the reference's reader then reuses the previous record's values: load it with the host "
                        "reader");
        }
        const int64_t stop = end == ~0ull ? ntok : (int64_t)(end >> 1);
        k_records<<<grid_of(ntok), kThreads, 0, s>>>(d_text, d_tok, ntok, d_head, d_val, stop, d_vrec, d_erec, d_cnt,
                                                     d_mm);
        LT_CK(cudaGetLastError(), "record launch");
        LT_CK(read(cnt, d_cnt, 16), "record counts");
    }
    int32_t mm[2] = {INT32_MAX, INT32_MIN};
    LT_CK(read(mm, d_mm, 8), "id range");
    const int64_t nv = (int64_t)cnt[0], ne = (int64_t)cnt[1];
    const int64_t range = nv + ne > 0 ? (int64_t)mm[1] - mm[0] + 1 : 0;
    if (range > ((int64_t)1 << 28)) {
        freeall();
        return fail(ctx, GSPAN_ERR_LIMIT, "vertex ids span more than 2^28 values (device loader)");
    }
    if (2 * ne > INT32_MAX) {
        freeall();
        return fail(ctx, GSPAN_ERR_LIMIT, "more than 2^31 directed edge entries");
    }
    // Dense vertex numbering in ascending id order.
    uint8_t* d_flag = nullptr;
    int32_t* d_rank = nullptr;
    LT_CK(alloc((void**)&d_flag, (size_t)range), "alloc id flags");
    LT_CK(alloc((void**)&d_rank, (size_t)range * 4), "alloc id ranks");
    int64_t n = 0;
    if (range > 0) {
        LT_CK(cudaMemsetAsync(d_flag, 0, (size_t)range, s), "clear id flags");
        k_id_flags<<<grid_of(nv + ne), kThreads, 0, s>>>(d_vrec, nv, d_erec, ne, mm[0], d_flag);
        const int64_t fb = (range + kChunk - 1) / kChunk;
        int64_t *d_fc = nullptr, *d_fo = nullptr;
        LT_CK(alloc((void**)&d_fc, (size_t)(fb + 1) * 8), "alloc id scan");
        LT_CK(alloc((void**)&d_fo, (size_t)(fb + 1) * 8), "alloc id scan");
        k_flag_count<<<(int)fb, kThreads, 0, s>>>(d_flag, range, d_fc);
        k_scan_small<<<1, 1024, 0, s>>>(d_fc, d_fo, fb);
        k_flag_rank<<<(int)fb, kThreads, 0, s>>>(d_flag, range, d_fo, d_rank);
        LT_CK(cudaGetLastError(), "id launches");
        LT_CK(read(&n, d_fo + fb, 8), "vertex count");
    }
    // Labels (last 'v' record wins, 0 when none) and the CSR.
    int32_t *d_vl = nullptr, *d_last = nullptr, *d_off = nullptr;
    int64_t *d_deg = nullptr, *d_off64 = nullptr;
    unsigned long long* d_cur = nullptr;
    gspan_edge* d_edges = nullptr;
    LT_CK(alloc((void**)&d_vl, (size_t)n * 4), "alloc labels");
    LT_CK(alloc((void**)&d_last, (size_t)n * 4), "alloc labels");
    LT_CK(alloc((void**)&d_deg, (size_t)(n + 1) * 8), "alloc degrees");
    LT_CK(alloc((void**)&d_off64, (size_t)(n + 2) * 8), "alloc offsets");
    LT_CK(alloc((void**)&d_off, (size_t)(n + 1) * 4), "alloc offsets");
    LT_CK(alloc((void**)&d_cur, (size_t)(n + 1) * 8), "alloc cursors");
    LT_CK(alloc((void**)&d_edges, (size_t)(2 * ne) * sizeof(gspan_edge)), "alloc edges");
    if (n > 0) {
        LT_CK(cudaMemsetAsync(d_vl, 0, (size_t)n * 4, s), "clear labels");
        LT_CK(cudaMemsetAsync(d_last, 0xFF, (size_t)n * 4, s), "clear labels");
        LT_CK(cudaMemsetAsync(d_deg, 0, (size_t)(n + 1) * 8, s), "clear degrees");
        k_vertex_labels<<<grid_of(nv), kThreads, 0, s>>>(d_vrec, nv, mm[0], d_rank, d_last, 0, d_vl);
        k_vertex_labels<<<grid_of(nv), kThreads, 0, s>>>(d_vrec, nv, mm[0], d_rank, d_last, 1, d_vl);
        k_degrees<<<grid_of(ne), kThreads, 0, s>>>(d_erec, ne, mm[0], d_rank, d_deg);
        // Offsets: exclusive scan of the n degrees (int64 scan, then int32).
        k_scan_small<<<1, 1024, 0, s>>>(d_deg, d_off64, n);
        k_offsets32<<<grid_of(n + 1), kThreads, 0, s>>>(d_off64, n + 1, d_off, d_cur);
        k_scatter_edges<<<grid_of(ne), kThreads, 0, s>>>(d_erec, ne, mm[0], d_rank, d_cur, d_edges);
        LT_CK(cudaGetLastError(), "graph launches");
    } else {
        LT_CK(cudaMemsetAsync(d_off, 0, 4, s), "clear offsets");
    }
    LT_CK(cudaStreamSynchronize(s), "text graph");
    const int32_t N = (int32_t)n, M = (int32_t)(2 * ne);
    const int32_t* offs[1] = {d_off};
    const int32_t* vls[1] = {d_vl};
    const gspan_edge* eds[1] = {d_edges};
    const gspan_status rc = upload_graphs(ctx, 1, &N, &M, offs, vls, eds, out, /*on_device=*/true);
    freeall();
#undef LT_CK
    if (rc == GSPAN_OK) {
        if (nr_nodes) *nr_nodes = N;
        if (nr_edges) *nr_edges = M;
    }
    return rc;
}

}  // namespace gs
