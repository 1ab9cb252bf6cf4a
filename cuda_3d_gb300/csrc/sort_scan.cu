// sort_scan.cu -- LSD radix sort of (uint64 key, int32 value) pairs and a device-wide
// exclusive scan, both single-pass per digit / per scan with decoupled look-back.
//
// The sort replaces the reference's thrust::sort_by_key calls
// (src/geometry/cuda_voxel_grid_down_sample.cu:136, src/geometry/cuda_nn_search.cu:581-582):
// it is stable, so equal keys keep ascending input (original index) order, which is
// the order the voxel sums and the neighbour scans are defined in.
//
// Every look-back wait is bounded: after the context's wait limit (polls, read from its
// control words when the kernel starts) the kernel records kErrTimeout in the context's
// error word and treats the missing state as the end of its look-back -- the partial
// prefix only lowers the offsets it writes, which stay inside the output -- so a
// scheduling fault shows up as a status, never as a hung GPU.
#include "internal.cuh"

namespace gca3d
{

constexpr int kSortThreads = 256;
constexpr int kSortItems = 12;
constexpr int kSortTile = kSortThreads * kSortItems; // 3072 keys per tile
constexpr int kSortWarps = kSortThreads / 32;
constexpr int kLookWindow = 8; // predecessor tiles read at once in the look-back

constexpr uint32_t kFlagAgg = 1u << 30;
constexpr uint32_t kFlagInc = 2u << 30;
constexpr uint32_t kFlagMask = 3u << 30;
constexpr uint32_t kCountMask = (1u << 30) - 1;

// Control words of one sort.  The keys come in P segments ([seg_off[s], seg_off[s+1]),
// the segment index being the key's most significant field, each segment's keys in
// ascending index order), so a segment's keys end up in its own range: the sort runs
// per segment -- digit offsets per segment, tiles that never straddle two segments,
// and a look-back that ends at the segment's first tile, so the look-back chains are
// as long as a segment, not as the batch.  A pass is skipped when every segment's
// keys share its digit (the segment field's digits always do).
struct SortCtl
{
    int nontrivial[8];
    int in_sel[8];
    uint32_t tile_ctr[8];
    uint32_t prep_ticket;
    int ntiles; // tiles over all segments
};

// per-segment scratch of a sort: hist[s][d][b] digit counts, doff[s][d][b] the first
// output position of bucket b of digit d in segment s, tile_first[s] the segment's
// first tile (P + 1 entries)
struct SortSeg
{
    uint32_t *hist;
    uint32_t *doff;
    int32_t *tile_first;
};

// a status word carries its flag and count together in one aligned 32-bit word, and
// nothing else is read on the strength of it, so publishing needs no release fence
__device__ __forceinline__ void st_relaxed(uint32_t *p, uint32_t v)
{
    asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
// a state word holds its flag and its count together, so a reader that uses only
// the word itself needs no ordering: relaxed loads, several in flight at once
__device__ __forceinline__ uint32_t ld_relaxed(const uint32_t *p)
{
    uint32_t v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release64(unsigned long long *p, unsigned long long v)
{
    asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ unsigned long long ld_acquire64(const unsigned long long *p)
{
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

// the byte-digit d of a sort word: bits [ks + 8 d, ks + 8 d + 8), ks the key's lowest bit
// (SortBuffers::d_kshift), zero above bit 63
__device__ __forceinline__ uint32_t sort_digit(uint64_t k, int ks, int d)
{
    const int sh = ks + 8 * d;
    return sh < 64 ? (uint32_t)(k >> sh) & 255u : 0u;
}

// per-segment histograms of all 8 byte-digits (block (x, s): segment s); also clears
// the first look-back status buffer
__global__ void k_sort_hist(const uint64_t *__restrict__ keys, const int32_t *seg_off, const int *d_kshift, SortSeg S,
                            uint32_t *status0, int64_t status_words)
{
    __shared__ uint32_t h[8][256];
    for (int i = threadIdx.x; i < 8 * 256; i += blockDim.x)
        (&h[0][0])[i] = 0;
    __syncthreads();
    const int seg = blockIdx.y;
    const int b = seg_off[seg], e = seg_off[seg + 1];
    const int ks = *d_kshift;
    for (int i = b + blockIdx.x * blockDim.x + threadIdx.x; i < e; i += gridDim.x * blockDim.x)
    {
        uint64_t k = keys[i];
#pragma unroll
        for (int d = 0; d < 8; ++d)
            atomicAdd(&h[d][sort_digit(k, ks, d)], 1u);
    }
    const int64_t nb = (int64_t)gridDim.x * gridDim.y, bid = (int64_t)blockIdx.y * gridDim.x + blockIdx.x;
    for (int64_t i = bid * blockDim.x + threadIdx.x; i < status_words; i += nb * blockDim.x)
        status0[i] = 0;
    __syncthreads();
    uint32_t *gh = S.hist + (size_t)seg * 8 * 256;
    for (int i = threadIdx.x; i < 8 * 256; i += blockDim.x)
    {
        uint32_t c = (&h[0][0])[i];
        if (c)
            atomicAdd(&gh[i], c);
    }
}

// per segment (block s): bucket offsets of every digit, whether the segment's digit
// varies, and its tile count; the last block: the segments' first tiles and the
// ping-pong bookkeeping.  One warp per digit, each lane scanning 8 consecutive buckets.
__global__ void k_sort_prep(SortCtl *ctl, SortSeg S, const int32_t *seg_off, int P, int npasses, int *d_sel)
{
    const int seg = blockIdx.x;
    const int b = seg_off[seg], n = seg_off[seg + 1] - b;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t *gh = S.hist + (size_t)seg * 8 * 256;
    uint32_t *go = S.doff + (size_t)seg * 8 * 256;
    for (int d = warp; d < npasses; d += blockDim.x >> 5)
    {
        uint32_t c[8], sum = 0;
        bool triv = n <= 1;
#pragma unroll
        for (int k = 0; k < 8; ++k)
        {
            c[k] = gh[d * 256 + 8 * lane + k];
            sum += c[k];
            triv |= (int)c[k] == n;
        }
        uint32_t incl = sum;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1)
        {
            const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o)
                incl += y;
        }
        uint32_t run = (uint32_t)b + incl - sum;
#pragma unroll
        for (int k = 0; k < 8; ++k)
        {
            go[d * 256 + 8 * lane + k] = run;
            run += c[k];
        }
        triv = __any_sync(0xffffffffu, triv);
        if (lane == 0 && !triv)
            atomicOr(&ctl->nontrivial[d], 1);
    }
    if (threadIdx.x == 0)
        S.tile_first[seg + 1] = (n + kSortTile - 1) / kSortTile;
    __shared__ int s_last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0)
        s_last = atomicAdd(&ctl->prep_ticket, 1u) == gridDim.x - 1;
    __syncthreads();
    if (!s_last)
        return;
    __threadfence();
    // exclusive prefix of the tile counts (P <= 4096: 16 per thread, then a block scan)
    __shared__ int s_part[256];
    constexpr int kPer = (kMaxSegments + 255) / 256;
    const int p0 = threadIdx.x * kPer;
    int cnt[kPer], sum = 0;
#pragma unroll
    for (int k = 0; k < kPer; ++k)
    {
        cnt[k] = p0 + k < P ? __ldcg(&S.tile_first[p0 + k + 1]) : 0;
        sum += cnt[k];
    }
    s_part[threadIdx.x] = sum;
    __syncthreads();
    if (threadIdx.x < 32)
    {
        int v[8], t = 0;
#pragma unroll
        for (int k = 0; k < 8; ++k)
        {
            v[k] = s_part[threadIdx.x * 8 + k];
            t += v[k];
        }
        int incl = t;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1)
        {
            const int y = __shfl_up_sync(0xffffffffu, incl, o);
            if ((int)threadIdx.x >= o)
                incl += y;
        }
        int run = incl - t;
#pragma unroll
        for (int k = 0; k < 8; ++k)
        {
            s_part[threadIdx.x * 8 + k] = run;
            run += v[k];
        }
    }
    __syncthreads();
    int run = s_part[threadIdx.x];
#pragma unroll
    for (int k = 0; k < kPer; ++k)
        if (p0 + k < P)
        {
            S.tile_first[p0 + k] = run;
            run += cnt[k];
        }
    if (threadIdx.x == 255)
    {
        // the last thread's running sum is the total
        ctl->ntiles = run;
        S.tile_first[P] = run;
    }
    if (threadIdx.x == 0)
    {
        int sel = 0;
        for (int d = 0; d < npasses; ++d)
        {
            ctl->in_sel[d] = sel;
            if (__ldcg(&ctl->nontrivial[d]))
                sel ^= 1;
        }
        *d_sel = sel;
    }
}

// the lanes of the warp whose value equals this lane's, for values below 512: one
// ballot per bit, each lane keeping the lanes that agree with it on every bit
__device__ __forceinline__ unsigned digit_peers(uint32_t d)
{
    unsigned m = 0xffffffffu;
#pragma unroll
    for (int b = 0; b < 9; ++b)
    {
        const bool bit = (d >> b) & 1u;
        const unsigned v = __ballot_sync(0xffffffffu, bit);
        m &= bit ? v : ~v;
    }
    return m;
}

// what one tile of a pass works on
struct TileJob
{
    uint32_t tile;
    int first, seg, seg_b, seg_e, tile_base, cnt, shift, pass;
    const uint64_t *kin;
    const int32_t *vin;
    uint64_t *kout;
    int32_t *vout;
    uint32_t *status;
};

// one tile of a pass: rank, stage in tile order, look back, scatter.  Packed keys carry
// their index, so that variant holds no value registers.
template <bool Packed>
__device__ __forceinline__ void sort_tile(const TileJob &J, SortCtl *ctl, const SortSeg &S, int *d_err,
                                          uint32_t (*s_whist)[256], uint32_t *s_excl, uint32_t *s_gbase,
                                          uint64_t *s_keys, int32_t *s_vals, uint32_t *s_wsum)
{
    const uint32_t tile = J.tile;
    const int first = J.first, seg = J.seg, tile_base = J.tile_base, cnt = J.cnt;
    [[maybe_unused]] const int seg_b = J.seg_b, seg_e = J.seg_e; // the checked build's index checks
    const int shift = J.shift, pass = J.pass;
    const uint64_t *kin = J.kin;
    const int32_t *vin = J.vin;
    uint64_t *kout = J.kout;
    int32_t *vout = J.vout;
    uint32_t *status = J.status;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const unsigned lt_mask = (1u << lane) - 1u;

    for (int i = threadIdx.x; i < kSortWarps * 256; i += kSortThreads)
        (&s_whist[0][0])[i] = 0;
    __syncthreads();

    uint64_t k[kSortItems];
    int32_t v[kSortItems];
    uint32_t rank[kSortItems];
    uint32_t dig4[kSortItems / 4] = {}; // the digits, four per word
    const int base = warp * 32 * kSortItems; // within the tile
#pragma unroll
    for (int it = 0; it < kSortItems; ++it)
    {
        const int idx = base + it * 32 + lane;
        k[it] = idx < cnt ? kin[tile_base + idx] : 0;
        v[it] = idx < cnt && !Packed ? vin[tile_base + idx] : 0;
        dig4[it / 4] |= ((uint32_t)(k[it] >> shift) & 255u) << (8 * (it % 4));
    }
    // warp-level stable ranking: the lanes holding the same digit (one ballot per digit
    // bit, a fixed cost, where a match instruction costs more the more distinct digits
    // the warp holds) read the warp's count of that digit, and the lowest of them adds
    // their number to it
#pragma unroll
    for (int it = 0; it < kSortItems; ++it)
    {
        const bool in = base + it * 32 + lane < cnt;
        const uint32_t d = (dig4[it / 4] >> (8 * (it % 4))) & 255u;
        const unsigned peers = digit_peers(in ? d : 256u);
        const uint32_t b = s_whist[warp][d];
        __syncwarp();
        if (in && (peers & lt_mask) == 0u)
            s_whist[warp][d] = b + __popc(peers);
        rank[it] = b + __popc(peers & lt_mask);
        __syncwarp();
    }
    __syncthreads();
    // per digit: prefix over warps, tile total
    const int t = threadIdx.x;
    uint32_t tot = 0;
#pragma unroll
    for (int w = 0; w < kSortWarps; ++w)
    {
        uint32_t c = s_whist[w][t];
        s_whist[w][t] = tot;
        tot += c;
    }
    // this tile's count of digit t, published for the segment's tiles after it
    uint32_t *st = status + (int64_t)tile * 256 + t;
    st_relaxed(st, (tile == first ? kFlagInc : kFlagAgg) | tot);
    // exclusive scan of the tile totals over digits (block scan of 256 values)
    uint32_t x = tot;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1)
    {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o)
            x += y;
    }
    if (lane == 31)
        s_wsum[warp] = x;
    __syncthreads();
    uint32_t wpre = 0;
    for (int w = 0; w < warp; ++w)
        wpre += s_wsum[w];
    const uint32_t tile_excl = wpre + x - tot;
    s_excl[t] = tile_excl;
    __syncthreads();
    // stage in tile-sorted order (needs only this tile's counts), so the keys leave
    // the registers before the look-back
#pragma unroll
    for (int it = 0; it < kSortItems; ++it)
    {
        if (base + it * 32 + lane < cnt)
        {
            const uint32_t d = (uint32_t)(k[it] >> shift) & 255u;
            const uint32_t pl = s_excl[d] + s_whist[warp][d] + rank[it];
            s_keys[pl] = k[it];
            if (!Packed)
                s_vals[pl] = v[it];
        }
    }
    // decoupled look-back across the segment's earlier tiles for digit t
    uint32_t excl = 0;
    if ((int)tile > first)
    {
        // the predecessors' states for this digit, kLookWindow at a time (independent
        // relaxed loads), consumed nearest first up to the nearest inclusive one (the
        // segment's first tile publishes an inclusive state at once)
        bool found = false;
        const uint32_t limit = wait_limit(d_err);
        for (int64_t p = (int64_t)tile - 1; p >= first && !found; p -= kLookWindow)
        {
            uint32_t s[kLookWindow];
#pragma unroll
            for (int j = 0; j < kLookWindow; ++j)
                s[j] = p - j >= first ? ld_relaxed(status + (p - j) * 256 + t) : kFlagInc;
#pragma unroll
            for (int j = 0; j < kLookWindow; ++j)
            {
                if (found)
                    break;
                uint32_t spins = 0;
                while ((s[j] & kFlagMask) == 0)
                {
                    if (++spins > limit)
                    {
                        atomicOr(d_err, kErrTimeout);
                        break;
                    }
                    if (spins > 64)
                        __nanosleep(64);
                    s[j] = ld_relaxed(status + (p - j) * 256 + t);
                }
                excl += s[j] & kCountMask;
                if ((s[j] & kFlagMask) != kFlagAgg)
                    found = true;
            }
        }
        st_relaxed(st, kFlagInc | (excl + tot));
    }
    s_gbase[t] = S.doff[((size_t)seg * 8 + pass) * 256 + t] + excl - tile_excl;
    __syncthreads();
    for (int j = threadIdx.x; j < cnt; j += kSortThreads)
    {
        uint64_t kk = s_keys[j];
        uint32_t d = (uint32_t)(kk >> shift) & 255u;
        uint32_t g = s_gbase[d] + j;
        if (!GCA_INDEX_OK((int)g - seg_b, seg_e - seg_b, d_err))
            continue;
        kout[g] = kk;
        if (!Packed)
            vout[g] = s_vals[j];
    }
}

__global__ void __launch_bounds__(kSortThreads, 4) k_sort_pass(
    uint64_t *keys0, int32_t *vals0, uint64_t *keys1, int32_t *vals1, SortCtl *ctl, SortSeg S,
    const int32_t *seg_off, int P, uint32_t *status_base, int64_t status_words, int pass, const int *d_ib,
    const int *d_kshift, int *d_err)
{
    __shared__ uint32_t s_whist[kSortWarps][256];
    __shared__ uint32_t s_excl[256];
    __shared__ uint32_t s_gbase[256];
    __shared__ uint64_t s_keys[kSortTile];
    __shared__ int32_t s_vals[kSortTile];
    __shared__ uint32_t s_tile;
    __shared__ int s_seg;
    __shared__ uint32_t s_wsum[kSortWarps];

    if (!ctl->nontrivial[pass])
        return;
    // the non-trivial passes alternate between two status buffers (as between the key
    // buffers): this pass clears the other one, which the previous non-trivial pass used
    // and the next one will use, so a trivial pass has nothing to clear
    const int sel = ctl->in_sel[pass];
    uint32_t *status = status_base + sel * status_words, *status_next = status_base + (sel ^ 1) * status_words;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < status_words;
         i += (int64_t)gridDim.x * blockDim.x)
        status_next[i] = 0;
    if (threadIdx.x == 0)
    {
        const uint32_t tk = atomicAdd(&ctl->tile_ctr[pass], 1u);
        // the segment of the tile: the last one whose first tile is <= tk (empty
        // segments share their first tile with the next one)
        int lo = 0, hi = P - 1;
        while (lo < hi)
        {
            const int mid = (lo + hi + 1) >> 1;
            if (S.tile_first[mid] <= (int)tk)
                lo = mid;
            else
                hi = mid - 1;
        }
        s_tile = tk;
        s_seg = lo;
    }
    __syncthreads();
    const uint32_t tile = s_tile;
    if ((int)tile >= ctl->ntiles)
        return;
    const int seg = s_seg;
    const int first = S.tile_first[seg];
    const int seg_b = seg_off[seg], seg_e = seg_off[seg + 1];
    const int tile_base = seg_b + ((int)tile - first) * kSortTile;
    const int cnt = min(kSortTile, seg_e - tile_base);
    const uint64_t *kin = sel ? keys1 : keys0;
    const int32_t *vin = sel ? vals1 : vals0;
    uint64_t *kout = sel ? keys0 : keys1;
    int32_t *vout = sel ? vals0 : vals1;
    // a non-trivial pass lies below bit 64 (the digits above are zero, so trivial)
    const int shift = *d_kshift + pass * 8;
    const TileJob J{tile, first, seg, seg_b, seg_e, tile_base, cnt, shift, pass, kin, vin, kout, vout, status};
    if (*d_ib != 0)
        sort_tile<true>(J, ctl, S, d_err, s_whist, s_excl, s_gbase, s_keys, s_vals, s_wsum);
    else
        sort_tile<false>(J, ctl, S, d_err, s_whist, s_excl, s_gbase, s_keys, s_vals, s_wsum);
}

int radix_sort(gca3d_context *ctx, SortBuffers &sb, const int32_t *seg_off, int P, int64_t cap, int64_t max_seg_cap,
               int max_bits)
{
    // four resident tiles per SM (47 KB of shared memory each) need the shared-memory side
    // of the L1 carveout
    static const bool carveout = cudaFuncSetAttribute(k_sort_pass, cudaFuncAttributePreferredSharedMemoryCarveout,
                                                      cudaSharedmemCarveoutMaxShared) == cudaSuccess;
    (void)carveout;
    if (P < 1 || P > kMaxSegments)
        return fail(ctx, GCA3D_ERR_INVALID_VALUE, "radix_sort: segment count");
    const int npasses = max_bits <= 0 ? 1 : (max_bits + 7) / 8;
    // tiles never straddle segments: at most one partial tile per segment more
    const int64_t ntiles = (cap + kSortTile - 1) / kSortTile + P;
    const int64_t status_words = ntiles * 256;
    SortCtl *ctl = ctx->arena.get<SortCtl>(1);
    uint32_t *status = ctx->arena.get<uint32_t>(2 * status_words);
    SortSeg S;
    S.hist = ctx->arena.get<uint32_t>((size_t)P * 8 * 256);
    S.doff = ctx->arena.get<uint32_t>((size_t)P * 8 * 256);
    S.tile_first = ctx->arena.get<int32_t>(P + 1);
    if (!ctl || !status || !sb.d_sel || !S.hist || !S.doff || !S.tile_first)
        return fail(ctx, GCA3D_ERR_OUT_OF_MEMORY, "radix_sort: scratch");
    GCA_CUDA(ctx, cudaMemsetAsync(ctl, 0, sizeof(SortCtl), ctx->stream));
    GCA_CUDA(ctx, cudaMemsetAsync(S.hist, 0, sizeof(uint32_t) * (size_t)P * 8 * 256, ctx->stream));
    // about 16 keys per thread in the largest segment (blocks past a smaller segment's end
    // return at once), so uneven segments do not leave one segment's blocks looping
    const int gx = (int)std::max<int64_t>(1, std::min<int64_t>(grid_for(max_seg_cap, kBlock * 16),
                                                               ((int64_t)ctx->num_sms * 32 + P - 1) / P));
    k_sort_hist<<<dim3(gx, P), kBlock, 0, ctx->stream>>>(sb.keys[0], seg_off, sb.d_kshift, S, status, status_words);
    GCA_CHECK_LAUNCH(ctx);
    // a trivial pass returns at once (conditional graph nodes around the passes, which
    // would skip the launch, measured slower: 13.4 against 13.0 ms per batch64 execute)
    k_sort_prep<<<P, 256, 0, ctx->stream>>>(ctl, S, seg_off, P, npasses, sb.d_sel);
    GCA_CHECK_LAUNCH(ctx);
    for (int p = 0; p < npasses; ++p)
    {
        GCA_PROF_BEGIN(ctx, kKidSortPass);
        k_sort_pass<<<(int)ntiles, kSortThreads, 0, ctx->stream>>>(sb.keys[0], sb.vals[0], sb.keys[1], sb.vals[1],
                                                                   ctl, S, seg_off, P, status, status_words, p,
                                                                   sb.d_ib, sb.d_kshift, ctx->d_err);
        GCA_CHECK_LAUNCH(ctx);
        GCA_PROF_END(ctx, kKidSortPass);
    }
    return GCA3D_OK;
}

// ---------------------------------------------------------------------------
// exclusive scan (int32), single pass with decoupled look-back
// ---------------------------------------------------------------------------
constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;
constexpr unsigned long long kSFlagAgg = 1ull << 62;
constexpr unsigned long long kSFlagInc = 2ull << 62;
constexpr unsigned long long kSFlagMask = 3ull << 62;
constexpr unsigned long long kSValMask = (1ull << 62) - 1;

struct ScanCtl
{
    uint32_t tile_ctr;
};

// warp 0 of a scan tile (all 32 lanes): publishes the tile's aggregate, looks back over
// the earlier tiles and publishes the inclusive prefix; returns the tile's exclusive
// prefix to every lane.  The 32 nearest predecessors' states are read at once (each
// wait bounded), the nearest inclusive one is found by ballot and the states up to it
// are summed across the warp; only a window of aggregates moves the look-back 32 tiles
// further.
__device__ __forceinline__ long long scan_lookback(int tile, long long agg, unsigned long long *status, int *d_err)
{
    const int lane = threadIdx.x & 31;
    unsigned long long *st = status + tile;
    long long excl = 0;
    if (lane == 0)
        st_release64(st, (tile == 0 ? kSFlagInc : kSFlagAgg) | (unsigned long long)agg);
    if (tile > 0)
    {
        for (int top = tile - 1;; top -= 32)
        {
            const int p = top - lane;
            unsigned long long s = kSFlagInc; // before tile 0: an inclusive zero
            if (p >= 0)
            {
                const uint32_t limit = wait_limit(d_err);
                uint32_t spins = 0;
                s = ld_acquire64(status + p);
                while ((s & kSFlagMask) == 0)
                {
                    if (++spins > limit)
                    {
                        atomicOr(d_err, kErrTimeout);
                        break;
                    }
                    if (spins > 64)
                        __nanosleep(64);
                    s = ld_acquire64(status + p);
                }
            }
            const unsigned inc = __ballot_sync(0xffffffffu, (s & kSFlagMask) != kSFlagAgg);
            const int stop = inc ? __ffs(inc) - 1 : 31;
            long long v = lane <= stop ? (long long)(s & kSValMask) : 0;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1)
                v += __shfl_xor_sync(0xffffffffu, v, o);
            excl += v;
            if (inc)
                break;
        }
        if (lane == 0)
            st_release64(st, kSFlagInc | (unsigned long long)(excl + agg));
    }
    return excl;
}

// what a scan reads and writes: item(i) is the value at i < n, put(i, e, v) receives
// the exclusive prefix e of item i (value v), total(t, n) the sum of all n items;
// bind() makes the copy a thread uses (device-side state read once)

struct ArrayScan
{
    const int32_t *in;
    int32_t *out;
    int32_t *d_total;
    __device__ ArrayScan bind() const { return *this; }
    __device__ int item(int64_t i) const { return in[i]; }
    __device__ void put(int64_t i, long long e, int) const { out[i] = (int32_t)e; }
    __device__ void total(long long t, int) const
    {
        if (d_total)
            *d_total = (int32_t)t;
    }
};

template <class Op>
__global__ void __launch_bounds__(kScanThreads) k_scan(const Op op_in, const int32_t *d_n, ScanCtl *ctl,
                                                       unsigned long long *status, int *d_err)
{
    const Op op = op_in.bind();
    __shared__ uint32_t s_tile;
    __shared__ long long s_wsum[kScanThreads / 32];
    __shared__ long long s_prefix;
    const int n = *d_n;
    const int ntiles = (n + kScanTile - 1) / kScanTile;
    if (threadIdx.x == 0)
        s_tile = atomicAdd(&ctl->tile_ctr, 1u);
    __syncthreads();
    const int tile = (int)s_tile;
    if (tile >= ntiles)
    {
        if (tile == 0 && threadIdx.x == 0)
            op.total(0, 0); // empty input
        return;
    }
    const int64_t base = (int64_t)tile * kScanTile + threadIdx.x * kScanItems;
    long long v[kScanItems];
    long long tsum = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i)
    {
        v[i] = base + i < n ? (long long)op.item(base + i) : 0;
        tsum += v[i];
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    long long x = tsum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1)
    {
        long long y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o)
            x += y;
    }
    if (lane == 31)
        s_wsum[warp] = x;
    __syncthreads();
    if (warp == 0)
    {
        long long agg = 0;
        for (int w = 0; w < kScanThreads / 32; ++w)
            agg += s_wsum[w];
        const long long excl = scan_lookback(tile, agg, status, d_err);
        if (lane == 0)
        {
            s_prefix = excl;
            if (tile == ntiles - 1)
                op.total(excl + agg, n);
        }
    }
    __syncthreads();
    long long run = s_prefix;
    for (int w = 0; w < warp; ++w)
        run += s_wsum[w];
    run += x - tsum;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i)
    {
        if (base + i < n)
            op.put(base + i, run, (int)v[i]);
        run += v[i];
    }
}

// the runs of equal keys of a sorted view in one pass: a tile's keys are read
// coalesced (thread t reads elements t, t + 256, ...), each element's run start (bit 0)
// and segment start (bit 1) go to shared memory as one byte, and every thread scans its
// own eight consecutive bytes; a run's exclusive prefix is its index, so starts[run] is
// its first position (starts[runs] = n) and seg_first[seg] the segment's first run
__global__ void __launch_bounds__(kScanThreads) k_run_scan(SortBuffers sb, const KeyLayout *lay, const int32_t *d_n,
                                                           ScanCtl *ctl, unsigned long long *status, int32_t *starts,
                                                           int32_t *seg_first, int32_t *d_runs, int *d_err)
{
    __shared__ uint32_t s_tile;
    __shared__ long long s_wsum[kScanThreads / 32];
    __shared__ long long s_prefix;
    __shared__ __align__(8) uint8_t s_f[kScanTile];
    const int n = *d_n;
    const int ntiles = (n + kScanTile - 1) / kScanTile;
    if (threadIdx.x == 0)
        s_tile = atomicAdd(&ctl->tile_ctr, 1u);
    __syncthreads();
    const int tile = (int)s_tile;
    if (tile >= ntiles)
    {
        if (tile == 0 && threadIdx.x == 0)
        {
            *d_runs = 0; // empty input
            starts[0] = 0;
        }
        return;
    }
    const SortedView sv = sorted_view(sb);
    const KeyLayout L = *lay;
    const int segshift = L.bx + L.by + L.bz;
    const int tbase = tile * kScanTile;
#pragma unroll
    for (int it = 0; it < kScanItems; ++it)
    {
        const int i = tbase + it * kScanThreads + (int)threadIdx.x;
        uint32_t f = 0;
        if (i < n)
        {
            if (i == 0)
                f = 3;
            else
            {
                const uint64_t k = sv.key(i), kp = sv.key(i - 1);
                f = (k != kp ? 1u : 0u) | (L.bseg && (k >> segshift) != (kp >> segshift) ? 2u : 0u);
            }
        }
        s_f[it * kScanThreads + threadIdx.x] = (uint8_t)f;
    }
    __syncthreads();
    const int base = tbase + (int)threadIdx.x * kScanItems;
    const uint64_t f8 = *reinterpret_cast<const uint64_t *>(&s_f[threadIdx.x * kScanItems]);
    const long long tsum = __popcll(f8 & 0x0101010101010101ull);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    long long x = tsum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1)
    {
        const long long y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o)
            x += y;
    }
    if (lane == 31)
        s_wsum[warp] = x;
    __syncthreads();
    if (warp == 0)
    {
        long long agg = 0;
        for (int w = 0; w < kScanThreads / 32; ++w)
            agg += s_wsum[w];
        const long long excl = scan_lookback(tile, agg, status, d_err);
        if (lane == 0)
        {
            s_prefix = excl;
            if (tile == ntiles - 1)
            {
                *d_runs = (int32_t)(excl + agg);
                starts[excl + agg] = n;
            }
        }
    }
    __syncthreads();
    long long run = s_prefix;
    for (int w = 0; w < warp; ++w)
        run += s_wsum[w];
    run += x - tsum;
#pragma unroll
    for (int j = 0; j < kScanItems; ++j)
    {
        const uint32_t f = (uint32_t)(f8 >> (8 * j)) & 3u;
        if (f & 1u)
        {
            starts[run] = base + j;
            if (f & 2u || base + j == 0)
                seg_first[L.bseg ? (int)(sv.key(base + j) >> segshift) : 0] = (int32_t)run;
            ++run;
        }
    }
}

int exclusive_scan(gca3d_context *ctx, const int32_t *in, int32_t *out, const int32_t *d_n,
                   int64_t cap, int32_t *d_total)
{
    const int64_t ntiles = (cap + kScanTile - 1) / kScanTile;
    ScanCtl *ctl = ctx->arena.get<ScanCtl>(1);
    unsigned long long *status = ctx->arena.get<unsigned long long>(ntiles > 0 ? ntiles : 1);
    if (!ctl || !status)
        return fail(ctx, GCA3D_ERR_OUT_OF_MEMORY, "exclusive_scan: scratch");
    GCA_CUDA(ctx, cudaMemsetAsync(ctl, 0, sizeof(ScanCtl), ctx->stream));
    GCA_CUDA(ctx, cudaMemsetAsync(status, 0, sizeof(unsigned long long) * (ntiles > 0 ? ntiles : 1), ctx->stream));
    k_scan<<<(int)(ntiles > 0 ? ntiles : 1), kScanThreads, 0, ctx->stream>>>(ArrayScan{in, out, d_total}, d_n, ctl,
                                                                             status, ctx->d_err);
    GCA_CHECK_LAUNCH(ctx);
    return GCA3D_OK;
}

int run_scan(gca3d_context *ctx, const SortBuffers &sb, const int32_t *d_n, int64_t cap, const KeyLayout *lay,
             int32_t *starts, int32_t *seg_first, int32_t *d_runs)
{
    const int64_t ntiles = (cap + kScanTile - 1) / kScanTile;
    ScanCtl *ctl = ctx->arena.get<ScanCtl>(1);
    unsigned long long *status = ctx->arena.get<unsigned long long>(ntiles > 0 ? ntiles : 1);
    if (!ctl || !status)
        return fail(ctx, GCA3D_ERR_OUT_OF_MEMORY, "run_scan: scratch");
    GCA_CUDA(ctx, cudaMemsetAsync(ctl, 0, sizeof(ScanCtl), ctx->stream));
    GCA_CUDA(ctx, cudaMemsetAsync(status, 0, sizeof(unsigned long long) * (ntiles > 0 ? ntiles : 1), ctx->stream));
    k_run_scan<<<(int)(ntiles > 0 ? ntiles : 1), kScanThreads, 0, ctx->stream>>>(sb, lay, d_n, ctl, status, starts,
                                                                                 seg_first, d_runs, ctx->d_err);
    GCA_CHECK_LAUNCH(ctx);
    return GCA3D_OK;
}

} // namespace gca3d

using namespace gca3d;

// A scan of `tiles` tiles launched with tiles - 1 blocks whose tile ticket starts at 1:
// tile 0 is never run, so status[0] is never published and tile 1's look-back waits
// on it until the wait limit; the later tiles wait on tile 1, which publishes after
// giving up.  Every block's tile lies in [1, tiles), every read and write inside the
// tiles * kScanTile inputs and outputs and the tiles status words.
int gca3d_selfcheck_wait(gca3d_context *ctx, int tiles, int polls, int *wait_status, double *elapsed_ms)
{
    if (!ctx || tiles < 2 || tiles > 64 || polls < 1 || !wait_status)
        return fail(ctx, GCA3D_ERR_INVALID_VALUE, "selfcheck_wait: tiles in 2..64, polls >= 1");
    cudaSetDevice(ctx->device);
    int old_limit = 0;
    int st = gca3d_get_wait_limit(ctx, &old_limit);
    if (st)
        return st;
    consume_device_error(ctx, "selfcheck_wait"); // start from a clear error word
    ctx->arena.reset();
    const int n = tiles * kScanTile;
    int32_t *in = ctx->arena.get<int32_t>(n), *out = ctx->arena.get<int32_t>(n);
    int32_t *d_n = ctx->arena.get<int32_t>(1);
    ScanCtl *ctl = ctx->arena.get<ScanCtl>(1);
    unsigned long long *status = ctx->arena.get<unsigned long long>(tiles);
    if (!in || !out || !d_n || !ctl || !status)
        return fail(ctx, GCA3D_ERR_OUT_OF_MEMORY, "selfcheck_wait: scratch");
    GCA_CUDA(ctx, cudaMemsetAsync(in, 0, sizeof(int32_t) * n, ctx->stream));
    GCA_CUDA(ctx, cudaMemsetAsync(status, 0, sizeof(unsigned long long) * tiles, ctx->stream));
    ctx->h_pinned[60] = n;
    ctx->h_pinned[61] = 1; // first ticket
    GCA_CUDA(ctx, cudaMemcpyAsync(d_n, ctx->h_pinned + 60, sizeof(int32_t), cudaMemcpyHostToDevice, ctx->stream));
    GCA_CUDA(ctx, cudaMemcpyAsync(&ctl->tile_ctr, ctx->h_pinned + 61, sizeof(uint32_t), cudaMemcpyHostToDevice,
                                  ctx->stream));
    st = gca3d_set_wait_limit(ctx, polls);
    if (st)
        return st;
    cudaEvent_t e0, e1;
    GCA_CUDA(ctx, cudaEventCreate(&e0));
    GCA_CUDA(ctx, cudaEventCreate(&e1));
    cudaEventRecord(e0, ctx->stream);
    k_scan<<<tiles - 1, kScanThreads, 0, ctx->stream>>>(ArrayScan{in, out, nullptr}, d_n, ctl, status, ctx->d_err);
    const cudaError_t le = cudaGetLastError();
    ctx->launches++;
    cudaEventRecord(e1, ctx->stream);
    const cudaError_t se = cudaStreamSynchronize(ctx->stream);
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (elapsed_ms)
        *elapsed_ms = ms;
    *wait_status = consume_device_error(ctx, "selfcheck_wait: scan");
    const int rs = gca3d_set_wait_limit(ctx, old_limit);
    if (le != cudaSuccess)
        return cuda_fail(ctx, le, "selfcheck_wait: launch");
    if (se != cudaSuccess)
        return cuda_fail(ctx, se, "selfcheck_wait: synchronize");
    return rs;
}
