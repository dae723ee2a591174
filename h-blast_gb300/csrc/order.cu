// order.cu -- the ordering pass and the database/lookup-hit counters.
//
// The word finder appends HSPs in whatever order warps finish; H-BLAST fixes
// its order on the host (memory_defrag, h_blast.cu:1160-1208).  Here a stable
// LSD radix sort on the device orders them by (query, subject, subject
// offset, query offset) -- per query and subject, the order in which NCBI's
// CPU word finder creates them (NF/blast_engine.c:553-576 feeds that list to
// BlastSaveInitHsp) -- and a gather writes the ordered records.  All sizes are
// read from device memory, so the pass needs no host round trip.
#include <cuda_runtime.h>

#include "kernels.h"

namespace hbg {

namespace {

constexpr int kSortThreads = 256;          // one thread per digit value
constexpr int kSortItems = 16;             // per thread per tile
constexpr int kSortTile = kSortThreads * kSortItems;

__device__ __forceinline__ int64_t live_count(const unsigned long long *count, int64_t cap) {
    unsigned long long n = *count;
    return (int64_t)(n < (unsigned long long)cap ? n : (unsigned long long)cap);
}

__device__ __forceinline__ unsigned lanemask_lt() {
    unsigned r;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(r));
    return r;
}

__global__ void make_keys(const hbg_hsp *in, const unsigned long long *count, int64_t cap,
                          uint64_t *keys, uint32_t *vals, int bs, int bso, int bqo) {
    const int64_t n = live_count(count, cap);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const hbg_hsp h = in[i];
        uint64_t k = (uint64_t)(uint32_t)h.query;
        k = (k << bs) | (uint64_t)(uint32_t)h.subject;
        k = (k << bso) | (uint64_t)(uint32_t)h.s_off;
        k = (k << bqo) | (uint64_t)(uint32_t)h.q_off;
        keys[i] = k;
        vals[i] = (uint32_t)i;
    }
}

// Per-tile digit histogram, stored digit-major: hist[d * nblk + b].
__global__ void __launch_bounds__(kSortThreads)
sort_histogram(const uint64_t *keys, const unsigned long long *count, int64_t cap, int shift,
               uint32_t *hist) {
    __shared__ uint32_t h[256];
    const int64_t n = live_count(count, cap);
    const int64_t nblk = (n + kSortTile - 1) / kSortTile;
    if (blockIdx.x >= nblk)
        return;
    h[threadIdx.x] = 0;
    __syncthreads();
    const int64_t base = (int64_t)blockIdx.x * kSortTile;
    for (int r = 0; r < kSortItems; ++r) {
        const int64_t i = base + (int64_t)r * kSortThreads + threadIdx.x;
        if (i < n)
            atomicAdd(&h[(keys[i] >> shift) & 255u], 1u);
    }
    __syncthreads();
    hist[(int64_t)threadIdx.x * nblk + blockIdx.x] = h[threadIdx.x];
}

// Exclusive scan of the 256 x nblk histogram in place (one CTA).
__global__ void __launch_bounds__(1024)
sort_scan(const unsigned long long *count, int64_t cap, uint32_t *hist) {
    __shared__ uint32_t part[1024];
    const int64_t n = live_count(count, cap);
    const int64_t nblk = (n + kSortTile - 1) / kSortTile;
    const int64_t total = nblk * 256;
    if (total == 0)
        return;
    const int64_t per = (total + blockDim.x - 1) / blockDim.x;
    const int64_t b0 = threadIdx.x * per;
    const int64_t b1 = b0 + per < total ? b0 + per : total;
    uint32_t sum = 0;
    for (int64_t i = b0; i < b1; ++i)
        sum += hist[i];
    part[threadIdx.x] = sum;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
        uint32_t t = threadIdx.x >= (unsigned)o ? part[threadIdx.x - o] : 0;
        __syncthreads();
        part[threadIdx.x] += t;
        __syncthreads();
    }
    uint32_t run = part[threadIdx.x] - sum;
    for (int64_t i = b0; i < b1; ++i) {
        uint32_t v = hist[i];
        hist[i] = run;
        run += v;
    }
}

// Stable scatter of one tile: elements keep their input order among equal
// digits (round-major, then warp, then lane).
__global__ void __launch_bounds__(kSortThreads)
sort_scatter(const uint64_t *kin, const uint32_t *vin, uint64_t *kout, uint32_t *vout,
             const unsigned long long *count, int64_t cap, int shift, const uint32_t *hist) {
    __shared__ uint32_t cnt[kSortThreads / 32][256];
    __shared__ uint32_t pre[kSortThreads / 32][256];
    __shared__ uint32_t run[256];
    __shared__ uint32_t rbase[256];
    __shared__ uint32_t gofs[256];
    const int64_t n = live_count(count, cap);
    const int64_t nblk = (n + kSortTile - 1) / kSortTile;
    if (blockIdx.x >= nblk)
        return;
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    run[t] = 0;
    gofs[t] = hist[(int64_t)t * nblk + blockIdx.x];
    for (int w = 0; w < kSortThreads / 32; ++w)
        cnt[w][t] = 0;
    __syncthreads();
    const int64_t base = (int64_t)blockIdx.x * kSortTile;
    for (int r = 0; r < kSortItems; ++r) {
        const int64_t i = base + (int64_t)r * kSortThreads + t;
        const bool valid = i < n;
        uint64_t k = 0;
        uint32_t v = 0;
        int dig = 256 + lane;  // unique non-digit for invalid lanes
        if (valid) {
            k = kin[i];
            v = vin[i];
            dig = (int)((k >> shift) & 255u);
        }
        const unsigned m = __match_any_sync(0xffffffffu, dig);
        const int rank = __popc(m & lanemask_lt());
        if (valid && rank == 0)
            cnt[warp][dig] = __popc(m);
        __syncthreads();
        {
            uint32_t acc = 0;
            for (int w = 0; w < kSortThreads / 32; ++w) {
                pre[w][t] = acc;
                acc += cnt[w][t];
                cnt[w][t] = 0;
            }
            rbase[t] = run[t];
            run[t] += acc;
        }
        __syncthreads();
        if (valid) {
            const uint32_t pos = gofs[dig] + rbase[dig] + pre[warp][dig] + (uint32_t)rank;
            kout[pos] = k;
            vout[pos] = v;
        }
        __syncthreads();
    }
}

__global__ void gather_hsps(const hbg_hsp *in, const uint32_t *vals,
                            const unsigned long long *count, int64_t cap, hbg_hsp *out) {
    const int64_t n = live_count(count, cap);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        out[i] = in[vals[i]];
}

// Per-query ranges of the ordered list (sorted by query, then subject):
// first[q] and end[q] bound query q's HSPs, passed[q] counts its subjects
// with at least one HSP.  All three start at zero.  Whole warps step
// together (warp-uniform loop) so the subject counts can be summed per warp
// and query before the atomic: the list is sorted, so a warp's lanes mostly
// share one query.
__global__ void query_ranges(const hbg_hsp *sorted, const unsigned long long *count, int64_t cap,
                             unsigned long long *first, unsigned long long *end,
                             unsigned long long *passed) {
    const int64_t n = live_count(count, cap);
    const int lane = threadIdx.x & 31;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t base = blockIdx.x * (int64_t)blockDim.x + (threadIdx.x - lane); base < n; base += stride) {
        const int64_t i = base + lane;
        const bool valid = i < n;
        int32_t q = -1;
        bool fresh = false;
        if (valid) {
            q = sorted[i].query;
            const int32_t s = sorted[i].subject;
            const bool new_q = i == 0 || sorted[i - 1].query != q;
            if (new_q)
                first[q] = (unsigned long long)i;
            if (i == n - 1 || sorted[i + 1].query != q)
                end[q] = (unsigned long long)(i + 1);
            fresh = new_q || sorted[i - 1].subject != s;
        }
        const unsigned same = __match_any_sync(0xffffffffu, q);
        const unsigned cnt = __popc(__ballot_sync(0xffffffffu, fresh) & same);
        if (valid && cnt && lane == __ffs(same) - 1)
            atomicAdd(passed + q, (unsigned long long)cnt);
    }
}

__global__ void __launch_bounds__(256)
db_histogram(const uint8_t *db, int64_t n, unsigned long long *hist) {
    extern __shared__ unsigned int hsm[];
    for (int i = threadIdx.x; i < HBG_NUM_CELLS; i += blockDim.x)
        hsm[i] = 0;
    __syncthreads();
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p + 2 < n;
         p += (int64_t)gridDim.x * blockDim.x) {
        const unsigned a = db[p], b = db[p + 1], c = db[p + 2];
        if (a && b && c)
            atomicAdd(&hsm[(a << 10) | (b << 5) | c], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < HBG_NUM_CELLS; i += blockDim.x)
        if (hsm[i])
            atomicAdd(hist + i, (unsigned long long)hsm[i]);
}

__global__ void __launch_bounds__(256)
query_hits(const unsigned long long *hist, const uint16_t *qcells, unsigned long long *out) {
    __shared__ unsigned long long part[256];
    const uint16_t *qc = qcells + (size_t)blockIdx.x * HBG_NUM_CELLS;
    unsigned long long acc = 0;
    for (int w = threadIdx.x; w < HBG_NUM_CELLS; w += blockDim.x)
        acc += hist[w] * (unsigned long long)qc[w];
    part[threadIdx.x] = acc;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < (unsigned)o)
            part[threadIdx.x] += part[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0)
        out[blockIdx.x] = part[0];
}

}  // namespace

int64_t order_max_blocks(int64_t cap) { return (cap + kSortTile - 1) / kSortTile; }

cudaError_t launch_order(const OrderArgs &a, cudaStream_t stream) {
    const int bits = a.bits_q + a.bits_s + a.bits_so + a.bits_qo;
    const int64_t maxblk = order_max_blocks(a.cap);
    if (maxblk == 0)
        return cudaSuccess;
    const int gblocks = (int)(maxblk * kSortItems < 65535 ? maxblk * kSortItems : 65535);
    make_keys<<<gblocks, 256, 0, stream>>>(a.in, a.count, a.cap, a.keys[0], a.vals[0],
                                           a.bits_s, a.bits_so, a.bits_qo);
    int src = 0;
    for (int shift = 0; shift < bits; shift += 8) {
        sort_histogram<<<(unsigned)maxblk, kSortThreads, 0, stream>>>(a.keys[src], a.count,
                                                                      a.cap, shift, a.hist);
        sort_scan<<<1, 1024, 0, stream>>>(a.count, a.cap, a.hist);
        sort_scatter<<<(unsigned)maxblk, kSortThreads, 0, stream>>>(
            a.keys[src], a.vals[src], a.keys[src ^ 1], a.vals[src ^ 1], a.count, a.cap, shift,
            a.hist);
        src ^= 1;
    }
    gather_hsps<<<gblocks, 256, 0, stream>>>(a.in, a.vals[src], a.count, a.cap, a.out);
    if (a.q_first)
        query_ranges<<<gblocks, 256, 0, stream>>>(a.out, a.count, a.cap, a.q_first, a.q_end, a.q_passed);
    return cudaGetLastError();
}

cudaError_t launch_db_histogram(const uint8_t *db, int64_t n, unsigned long long *hist,
                                cudaStream_t stream) {
    const size_t smem = HBG_NUM_CELLS * sizeof(unsigned int);
    cudaError_t e = cudaFuncSetAttribute(db_histogram, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess)
        return e;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    db_histogram<<<sms > 0 ? sms : 1, 256, smem, stream>>>(db, n, hist);
    return cudaGetLastError();
}

cudaError_t launch_query_hits(const unsigned long long *hist, const uint16_t *query_cells,
                              int32_t n_queries, unsigned long long *out, cudaStream_t stream) {
    if (n_queries <= 0)
        return cudaSuccess;
    query_hits<<<n_queries, 256, 0, stream>>>(hist, query_cells, out);
    return cudaGetLastError();
}

}  // namespace hbg
