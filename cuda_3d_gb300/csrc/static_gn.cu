// static_gn.cu -- the Gauss-Newton system of given correspondences, computed without
// any device allocation.
//
// Who needs this: a caller that cannot allocate device memory once it is running.
// Two common cases: a real-time capture loop that must not stall, and cudaMalloc
// synchronises the whole device and can take milliseconds; and a host application
// whose own memory manager has already claimed the GPU's memory and gives this library
// only the buffers it filled itself.  gca3d_build_gauss_newton (the regular entry
// point) takes cloud handles and draws its scratch from a context arena, both of which
// allocate.  gca3d_build_gauss_newton_static takes plain device pointers and a stream
// and keeps its scratch -- one FP64 partial sum per block, the point count and the
// last-block ticket -- in g_gn_scratch below, a fixed array that every GPU which
// loads this library holds until the process exits.
#include "icp.cuh"

#include <mutex>

namespace
{

using namespace gca3d;

constexpr int kStaticBlocks = 2048;          // partial sums available
constexpr int kStaticChunk = 4096;           // source points per block
constexpr int64_t kStaticMaxPoints = (int64_t)kStaticBlocks * kStaticChunk; // 8,388,608
constexpr int kMaxDevices = 64;

struct StaticScratch
{
    double partials[kStaticBlocks * kTermsPad]; // 512 KiB
    double out[kTermsPad];
    int32_t n_src;
    unsigned ticket;
};

static __device__ __align__(256) StaticScratch g_gn_scratch;

std::mutex g_setup_mutex;
StaticScratch *g_scratch_addr[kMaxDevices] = {};

// device address of g_gn_scratch on the current device, looked up once per device
int scratch_on_current_device(StaticScratch **out)
{
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
    {
        cudaGetLastError();
        return GCA3D_ERR_CUDA;
    }
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_addr[dev])
    {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_gn_scratch);
        if (e != cudaSuccess || !p)
        {
            cudaGetLastError();
            return GCA3D_ERR_CUDA;
        }
        g_scratch_addr[dev] = static_cast<StaticScratch *>(p);
    }
    *out = g_scratch_addr[dev];
    return GCA3D_OK;
}

// the count the kernel reads and a zero ticket; the partials need no clearing
// (each block writes its own before the last block reads them)
__global__ void k_static_prepare(StaticScratch *s, int32_t n)
{
    s->n_src = n;
    s->ticket = 0u;
}

// 21 upper JTJ terms + 6 JTr + r^2 -> row-major 6x6, 6-vector, scalar
__global__ void k_static_expand(const StaticScratch *s, double *jtj, double *jtr, double *r2)
{
    const int t = threadIdx.x;
    if (t < 36)
    {
        int a = t / 6, b = t % 6;
        if (a > b)
        {
            int x = a;
            a = b;
            b = x;
        }
        const int u = a * 6 - a * (a - 1) / 2 + (b - a);
        jtj[t] = s->out[u];
    }
    if (t < 6)
        jtr[t] = s->out[21 + t];
    if (t == 0)
        *r2 = s->out[27];
}

} // namespace

extern "C" int gca3d_build_gauss_newton_static(void *stream, const void *src_pos, int32_t n_src,
                                               const void *tgt_pos, const void *tgt_nrm, const void *tgt_grd,
                                               const int32_t *nn, float lambda, double *jtj, double *jtr,
                                               double *r2)
{
    if (n_src < 0 || (n_src > 0 && (!src_pos || !nn)) || !tgt_pos || !tgt_nrm || !tgt_grd || !jtj || !jtr || !r2)
        return GCA3D_ERR_INVALID_VALUE;
    if (!(lambda >= 0.0f && lambda <= 1.0f))
        return GCA3D_ERR_INVALID_VALUE;
    if ((int64_t)n_src > kStaticMaxPoints)
        return GCA3D_ERR_CAPACITY;
    StaticScratch *s = nullptr;
    const int st = scratch_on_current_device(&s);
    if (st)
        return st;
    cudaStream_t cs = (cudaStream_t)stream;
    const int blocks = n_src > 0 ? (int)((n_src + kStaticChunk - 1) / kStaticChunk) : 1;
    k_static_prepare<<<1, 1, 0, cs>>>(s, n_src);
    k_build_gn<<<blocks, kIcpThreads, 0, cs>>>(
        static_cast<const float4 *>(src_pos), &s->n_src, static_cast<const float4 *>(tgt_pos),
        static_cast<const float4 *>(tgt_nrm), static_cast<const float4 *>(tgt_grd), nn, sqrtf(lambda),
        sqrtf(1.0f - lambda), s->partials, &s->ticket, s->out, nullptr, nullptr);
    k_static_expand<<<1, 64, 0, cs>>>(s, jtj, jtr, r2);
    if (cudaGetLastError() != cudaSuccess)
        return GCA3D_ERR_CUDA;
    return GCA3D_OK;
}
