// internal.cuh -- shared types and device helpers of the gca3d library.
#pragma once

#include "gca3d.h"

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <utility>
#include <vector>

namespace gca3d
{

// ---------------------------------------------------------------------------
// limits
// ---------------------------------------------------------------------------
constexpr int kMaxSegments = 4096;       // pairs / clouds in one batched stage
constexpr int kBlock = 256;              // threads per block for streaming kernels
constexpr int kWaitLimitDefault = 1 << 22; // polls before a cross-block wait gives up (about 0.3 s)

// device error word bits
enum : int
{
    kErrTimeout = 1,
    kErrCapacity = 2,
    kErrKeyBits = 4,
    kErrSingular = 8,
    kErrInvalid = 16,
    kErrBounds = 32, // an index check of the checked build failed
};

// Index checks of the checked build (compiled with -DGCA3D_CHECKED, the library
// libgca3d_checked.so): an index outside [0, n) sets kErrBounds in the context's error
// word and the access is skipped, so a bad index becomes a status, never a fault or a
// trap.  In the regular build the checks compile to nothing (n is not evaluated).
#ifdef GCA3D_CHECKED
#define GCA_INDEX_OK(i, n, err) ::gca3d::index_ok((long long)(i), (long long)(n), (err))
#else
#define GCA_INDEX_OK(i, n, err) true
#endif

// ---------------------------------------------------------------------------
// scratch memory: chunked bump allocator, reset per top-level call.  A replay
// of the same sequence of requests returns the same addresses, which is what
// graph capture relies on.
// ---------------------------------------------------------------------------
struct Arena
{
    struct Chunk
    {
        char *ptr = nullptr;
        size_t size = 0, used = 0;
    };
    std::vector<Chunk> chunks;
    size_t cur = 0;
    bool frozen = false; // no growth allowed (during capture)
    bool failed = false;

    void *take(size_t bytes);
    void reset()
    {
        for (auto &c : chunks)
            c.used = 0;
        cur = 0;
        failed = false;
    }
    void release();
    void swap(Arena &o)
    {
        chunks.swap(o.chunks);
        std::swap(cur, o.cur);
        std::swap(frozen, o.frozen);
        std::swap(failed, o.failed);
    }
    Arena() = default;
    Arena(const Arena &) = delete;
    Arena &operator=(const Arena &) = delete;
    ~Arena() { release(); }
    template <typename T> T *get(size_t count) { return static_cast<T *>(take(count * sizeof(T))); }
};

} // namespace gca3d

// ---------------------------------------------------------------------------
// opaque handles
// ---------------------------------------------------------------------------
namespace gca3d
{
enum KernelId : int
{
    kKidNone = -1,
    kKidIcpIter = 0,
    kKidSortPass,
    kKidNormals,
    kKidVoxelReduce,
    kKidGridScatter,
    kKidFrame,
    kKidCount
};
struct Profiler
{
    int target = kKidNone;
    std::vector<cudaEvent_t> events; // start/stop pairs
    size_t used = 0;
};
} // namespace gca3d

struct gca3d_context
{
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int num_sms = 0;
    gca3d::Arena arena;
    // device control words: [0] error bits (kErr*, set with atomicOr by kernels and
    // consumed by the host), [1] polls after which a cross-block wait gives up
    // (gca3d_set_wait_limit; kernels read it when they start)
    int *d_err = nullptr;
    int *h_pinned = nullptr; // pinned scratch for small read-backs (64 ints)
    int upload_mode = 0;     // GCA3D_UPLOAD_IN_PLACE or GCA3D_UPLOAD_COPY_ENGINE
    int64_t launches = 0;
    std::string last_error;
    gca3d::Profiler prof;
};

struct gca3d_cloud
{
    int64_t capacity = 0;
    float4 *pos = nullptr; // x, y, z, intensity
    float4 *col = nullptr; // r, g, b, 0
    float4 *nrm = nullptr;
    float4 *grd = nullptr;
    int32_t *d_count = nullptr;
    bool has_normals = false;
    bool has_grad = false;
    float grad_radius = 0.0f;
    int device = 0;
};

namespace gca3d
{

// ---------------------------------------------------------------------------
// host helpers
// ---------------------------------------------------------------------------
int fail(gca3d_context *ctx, int status, const std::string &msg);
int cuda_fail(gca3d_context *ctx, cudaError_t e, const char *where);
#define GCA_CUDA(ctx, call)                                                                        \
    do                                                                                             \
    {                                                                                              \
        cudaError_t e_ = (call);                                                                   \
        if (e_ != cudaSuccess)                                                                     \
            return ::gca3d::cuda_fail((ctx), e_, #call);                                           \
    } while (0)
#define GCA_CHECK_LAUNCH(ctx)                                                                      \
    do                                                                                             \
    {                                                                                              \
        (ctx)->launches++;                                                                         \
        cudaError_t e_ = cudaGetLastError();                                                       \
        if (e_ != cudaSuccess)                                                                     \
            return ::gca3d::cuda_fail((ctx), e_, __func__);                                        \
    } while (0)

// event bracket around launches of the profiled kernel (no-op otherwise)
void prof_mark(gca3d_context *ctx, int kid);
#define GCA_PROF_BEGIN(ctx, kid) ::gca3d::prof_mark((ctx), (kid))
#define GCA_PROF_END(ctx, kid) ::gca3d::prof_mark((ctx), (kid))

inline int div_up(int64_t a, int64_t b) { return (int)((a + b - 1) / b); }
inline int grid_for(int64_t n, int per_block = kBlock)
{
    int g = div_up(n > 0 ? n : 1, per_block);
    return g > 0 ? g : 1;
}
int ensure_attr(gca3d_context *ctx, gca3d_cloud *c, bool normals, bool grad);
// reads and clears the device error word; maps bits to a status
int consume_device_error(gca3d_context *ctx, const char *where);
// the status for an error word already read back (0: GCA3D_OK)
int device_error_status(gca3d_context *ctx, int word, const char *where);

// ---------------------------------------------------------------------------
// device helpers
// ---------------------------------------------------------------------------

// colour -> intensity in FP64 then rounded, without contraction, as
// color3::to_intensity (src/geometry/type.hpp:45-51)
__device__ __forceinline__ float intensity_of(float r, float g, float b)
{
    double s = __dadd_rn(__dmul_rn(0.2126, (double)r), __dmul_rn(0.7152, (double)g));
    s = __dadd_rn(s, __dmul_rn(0.0722, (double)b));
    return (float)s;
}

// float <-> order-preserving int (for atomicMin/atomicMax on floats)
__device__ __forceinline__ int float_to_ordered(float f)
{
    int i = __float_as_int(f);
    return i >= 0 ? i : i ^ 0x7FFFFFFF;
}
__device__ __forceinline__ float ordered_to_float(int i) { return __int_as_float(i >= 0 ? i : i ^ 0x7FFFFFFF); }
inline float ordered_to_float_host(int i)
{
    int j = i >= 0 ? i : i ^ 0x7FFFFFFF;
    float f;
    memcpy(&f, &j, 4);
    return f;
}

// squared distance q - p, unfused, the reference's order (cuda_nn_search.cu:195-200)
__device__ __forceinline__ float dist2_ref(float qx, float qy, float qz, float px, float py, float pz)
{
    float dx = __fsub_rn(qx, px), dy = __fsub_rn(qy, py), dz = __fsub_rn(qz, pz);
    return __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
}

// floor((p - mn) / cell), IEEE sub and div (cuda_voxel_grid_down_sample.cu:40-45)
__device__ __forceinline__ int cell_of(float p, float mn, float cell)
{
    return __float2int_rd(__fdiv_rn(__fsub_rn(p, mn), cell));
}

__device__ __forceinline__ int bitlen_u32(uint32_t v) { return v ? 32 - __clz(v) : 0; }

// block-wide min/max of 3 components, then one atomic per component per block
// (per-warp atomics on the same few words serialise in one L2 slice)
__device__ __forceinline__ void block_bounds_commit(float mn[3], float mx[3], int *ord6)
{
    __shared__ float s_mn[3][32], s_mx[3][32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
        {
            mn[a] = fminf(mn[a], __shfl_xor_sync(0xffffffffu, mn[a], o));
            mx[a] = fmaxf(mx[a], __shfl_xor_sync(0xffffffffu, mx[a], o));
        }
    if (lane == 0)
        for (int a = 0; a < 3; ++a)
            s_mn[a][warp] = mn[a], s_mx[a][warp] = mx[a];
    __syncthreads();
    if (threadIdx.x < 3)
    {
        const int a = threadIdx.x;
        float m = s_mn[a][0], M = s_mx[a][0];
        for (int w = 1; w < nw; ++w)
            m = fminf(m, s_mn[a][w]), M = fmaxf(M, s_mx[a][w]);
        atomicMin(ord6 + a, float_to_ordered(m));
        atomicMax(ord6 + 3 + a, float_to_ordered(M));
    }
}

template <typename T> __device__ __forceinline__ T warp_sum(T v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// the wait limit of the context whose control words ctl points to (see gca3d_context)
__device__ __forceinline__ uint32_t wait_limit(const int *ctl)
{
    return (uint32_t)*(const volatile int *)(ctl + 1);
}

__device__ __forceinline__ bool index_ok(long long i, long long n, int *err)
{
    if (i >= 0 && i < n)
        return true;
    atomicOr(err, kErrBounds);
    return false;
}

// bounded spin read of a volatile 64-bit status word until pred holds
__device__ __forceinline__ unsigned long long ld_volatile_u64(const unsigned long long *p)
{
    return *reinterpret_cast<const volatile unsigned long long *>(p);
}

// ---------------------------------------------------------------------------
// batched ("segmented") point sets: P clouds back to back
// ---------------------------------------------------------------------------

// per-segment AABB as ordered ints: [seg][0..2] min, [seg][3..5] max
struct SegBounds
{
    int *ord; // 6 * P
};

// parameters of one packed 64-bit cell key layout, shared by all segments
struct KeyLayout
{
    int bseg, bx, by, bz; // bits per field; key = seg|cx|cy|cz from MSB to LSB
    int total_bits;
    int morton; // voxel keys only: seg | bit-interleaved (cx, cy, cz), bx = by = bz
};

// one open-addressing slot of the row hash: the key and the row's [start, end) in
// the sorted arrays, read with a single 16-byte load
struct __align__(16) RowSlot
{
    unsigned long long key;
    int start;
    int end;
};

// a grid over the target segments
struct GridDev
{
    // per segment
    float3 *gmin;  // grid origin
    float cell;     // cell edge
    float inv_cell; // 1 / cell (conservative bounds only; cells are assigned by division)
    KeyLayout *layout;
    // sorted points (global positions over all segments)
    float4 *spos;  // x, y, z, __int_as_float(cz)
    int32_t *sidx; // batch index of the point (original order)
    float *sint;   // intensity in sorted order
    int *scz;      // z cell in sorted order (compact copy for the in-row binary search)
    uint64_t *skey;
    // row hash: key = (seg, cx, cy) -> [start, end) in one 16-byte slot; at least
    // twice as many slots as points, so the first probe nearly always decides
    RowSlot *slots;
    uint32_t hmask;
    const int32_t *seg_off; // [P + 1] offsets of the segments in the sorted arrays
    const int32_t *d_n;     // points in the grid (seg_off[P])
    int *err;               // the context's error word (index checks of the checked build)
};

constexpr unsigned long long kEmptyKey = ~0ull;

__device__ __forceinline__ uint32_t hash_u64(unsigned long long k)
{
    k ^= k >> 33;
    k *= 0xff51afd7ed558ccdull;
    k ^= k >> 33;
    k *= 0xc4ceb9fe1a85ec53ull;
    k ^= k >> 33;
    return (uint32_t)k;
}

__device__ __forceinline__ ulonglong2 slot_load(const RowSlot *slots, uint32_t h)
{
    return __ldg(reinterpret_cast<const ulonglong2 *>(slots + h));
}

// continue a linear probe after the first slot missed
static __device__ __noinline__ int2 row_probe_rest(const RowSlot *slots, uint32_t hmask, unsigned long long rk, uint32_t h)
{
    for (uint32_t probe = 1; probe <= hmask; ++probe)
    {
        h = (h + 1) & hmask;
        const ulonglong2 v = slot_load(slots, h);
        if (v.x == rk)
            return make_int2((int)(uint32_t)v.y, (int)(uint32_t)(v.y >> 32));
        if (v.x == kEmptyKey)
            break;
    }
    return make_int2(0, 0);
}

// ---------------------------------------------------------------------------
// stage entry points implemented in the .cu files (all stream-ordered)
// ---------------------------------------------------------------------------

// radix sort of (key, value) pairs by the low `max_bits` bits, n on the device.
// keys/vals are ping-pong buffers of capacity `cap`; on return *result_in_alt
// (device int) says whether the sorted data is in the alternate buffers.
// A sort of (key, index) pairs runs in one of two forms, chosen on the device by the
// kernel that writes the keys, once the key layout is known: packed, (key << ib) |
// index in one 64-bit word, when the key's bits and ib (the bits of the largest index)
// fit in 64 -- 8 bytes per element each way per pass instead of 12 -- or keys and
// indices in separate arrays.  The index is the element's position when the keys are
// written, so in both forms equal keys keep ascending index order.
struct SortBuffers
{
    uint64_t *keys[2];
    int32_t *vals[2];
    int *d_sel;    // device: index of the buffer holding the sorted data
    int *d_ib;     // device: index bits of the packed form, 0 for separate arrays
    int *d_kshift; // device: the key's lowest bit in a sort word (ib, plus sub-cell bits a
                   // voxel stage carries for finer scales); the digits start there
};

// index bits of a sort of at most cap elements
inline int index_bits(int64_t cap)
{
    int b = 1;
    while ((1ll << b) < cap)
        ++b;
    return b;
}

// the packed form's index bits for a key of key_bits bits, or 0 when it does not fit
__device__ __forceinline__ int packed_index_bits(int key_bits, int ib) { return key_bits + ib <= 64 ? ib : 0; }

// element i of the key kernels' output: the word w (the key, with any sub-cell bits
// below it) and index i
__device__ __forceinline__ void sort_store(uint64_t *keys, int32_t *vals, int i, uint64_t w, int ib)
{
    if (ib)
        keys[i] = (w << ib) | (uint64_t)(uint32_t)i;
    else
    {
        keys[i] = w;
        vals[i] = i;
    }
}

// the sorted keys and indices, whichever the form
struct SortedView
{
    const uint64_t *k;
    const int32_t *v;
    int ib, kshift;
    __device__ __forceinline__ uint64_t key(int i) const { return k[i] >> kshift; }
    __device__ __forceinline__ int32_t val(int i) const
    {
        return ib ? (int32_t)(k[i] & ((1ull << ib) - 1ull)) : v[i];
    }
};
__device__ __forceinline__ SortedView sorted_view(const SortBuffers &sb)
{
    const int sel = *sb.d_sel;
    return SortedView{sb.keys[sel], sb.vals[sel], *sb.d_ib, *sb.d_kshift};
}

// stable LSD sort of the keys in sb.keys[0] (and sb.vals[0]) in place, segment by
// segment: seg_off[P + 1] (device) holds the segments' element ranges, at most cap
// elements in all and max_seg_cap in one segment; the segment index must be the keys'
// most significant field
int radix_sort(gca3d_context *ctx, SortBuffers &sb, const int32_t *seg_off, int P, int64_t cap, int64_t max_seg_cap,
               int max_bits);

// exclusive scan of int32 values (n on the device), writes total to *d_total
int exclusive_scan(gca3d_context *ctx, const int32_t *in, int32_t *out, const int32_t *d_n,
                   int64_t cap, int32_t *d_total);
// the runs of equal keys of a sorted view in one scan: starts[r] the first position of
// run r, starts[runs] = n, *d_runs the number of runs, seg_first[s] the first run of
// segment s (left untouched, e.g. -1, for an empty segment)
int run_scan(gca3d_context *ctx, const SortBuffers &sb, const int32_t *d_n, int64_t cap, const KeyLayout *lay,
             int32_t *starts, int32_t *seg_first, int32_t *d_runs);

} // namespace gca3d
