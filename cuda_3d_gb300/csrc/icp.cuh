// icp.cuh -- per-pair device state and per-scale parameters of the ICP kernels.
#pragma once

#include "grid_query.cuh"
#include "stages.cuh"

namespace gca3d
{

constexpr int kIcpThreads = 256;
constexpr int kIcpChunk = 1024; // source points per accumulate work item (one partial each)
constexpr int kNNChunk = 256;   // default source points per correspondence work item
constexpr int kNNChunkMin = 64; // the smallest item size a tuning may choose
constexpr int kNNChunkMax = 512; // the largest

// the launch shape in force (defaults filled in)
struct IcpShape
{
    int nn_chunk = kNNChunk;
    int nn_bps = 10;
    int acc_bps = 6;
    bool fused = false; // the accumulate's last block of each pair finalizes it
};
IcpShape icp_shape(const gca3d_tuning &t);
constexpr int kTerms = 30;      // 21 JTJ (upper) + 6 JTr + r^2 + correspondences + sum d^2
constexpr int kTermsPad = 32;

struct PairState
{
    double T[16];
    double rmse_ref, fitness, inlier_rmse;
    int iters;
    int converged;
    int active;
    int status;
    unsigned int ticket;
    int nblocks;    // accumulate work items (kIcpChunk points) of the scale
    int nblocks_nn; // correspondence work items (kNNChunk points) of the scale
    int nsrc;
    int ntgt;
    int scale;
    int nn_warm; // the correspondences of the previous iteration of this scale are valid
    int scale_iters[GCA3D_MAX_SCALES];
    int scale_nsrc[GCA3D_MAX_SCALES];
    int scale_ntgt[GCA3D_MAX_SCALES];
};

// what the finalize of an iteration saw: the pose it started from, the summed
// system and the step (recorded for the adjoint of unrolled iterations)
struct IcpTrace
{
    double T[16];
    double S[kTerms];
    double x[6];
    int status;
    int pad;
};

struct IcpScale
{
    float max_corr;
    float sqrt_lg, sqrt_lc;
    int update_map;
    double rot_eps, trans_eps;
    IcpTrace *trace = nullptr; // [trace_cap iterations][P pairs] or null
    int trace_cap = 0;
};

// control of one iteration: each finalized pair takes a ticket (zero before the
// first iteration); the last one rebuilds the work maps and, in a captured
// schedule (iter set), counts the iteration and sets the WHILE node's condition.
// The maps are bmap[P + 2] (item offsets, total, active pairs) and bmap_nn[P + 2]
// (item offsets, total, work queue).
struct IcpLoop
{
    cudaGraphConditionalHandle handle = 0;
    int *iter = nullptr;
    unsigned *ticket = nullptr;
    int max_iter = 0;
};

// the Gauss-Newton system for given correspondences (defined in icp.cu); the block
// partials, the ticket and the count are scratch supplied by the caller.  With d_nt
// (the target count) an index at or beyond it is skipped and recorded as kErrInvalid
// in *d_err; without it the indices must lie inside the target.
__global__ void __launch_bounds__(kIcpThreads)
    k_build_gn(const float4 *__restrict__ sp, const int32_t *d_ns, const float4 *__restrict__ tp,
               const float4 *__restrict__ tn, const float4 *__restrict__ tg, const int32_t *nn, float slg, float slc,
               double *partials, unsigned *ticket, double *out, const int32_t *d_nt, int *d_err);

int icp_state_init(gca3d_context *ctx, PairState *st, int P, const double *d_Tinit);
int icp_setup(gca3d_context *ctx, PairState *st, int P, const int32_t *src_off, const int32_t *tgt_off, int *bmap,
              int *bmap_nn, int scale, int nn_chunk);
int icp_iteration(gca3d_context *ctx, const Batch &src, const Grid &g, const float4 *attr0, const float4 *attr1,
                  PairState *st, int *bmap, int max_blocks, int *bmap_nn, int max_blocks_nn, double *partials,
                  int2 *corr, const NNCerts &cert, const IcpScale &prm, bool compensated, int32_t *nn_out,
                  const IcpLoop &loop, const IcpShape &shape);
// the two halves of an iteration: the correspondence search (skipped on the device when
// guard is given and its iteration count has reached the budget), and the accumulation
// with the solve and pose update
int icp_search(gca3d_context *ctx, const Batch &src, const Grid &g, PairState *st, int *bmap_nn, int max_blocks_nn,
               int2 *corr, const NNCerts &cert, const IcpScale &prm, int32_t *nn_out, const IcpLoop *guard,
               const IcpShape &shape);
int icp_update(gca3d_context *ctx, const Batch &src, const Grid &g, const float4 *attr0, const float4 *attr1,
               PairState *st, int *bmap, int max_blocks, int *bmap_nn, double *partials, const int2 *corr,
               const IcpScale &prm, bool compensated, const IcpLoop &loop, const IcpShape &shape);
int build_gn(gca3d_context *ctx, const gca3d_cloud *src, const gca3d_cloud *tgt, const int32_t *nn, float lambda,
             double *out30);
int abs_residual(gca3d_context *ctx, const gca3d_cloud *src, const gca3d_cloud *tgt, const int32_t *nn, float lambda,
                 float *out);

} // namespace gca3d
