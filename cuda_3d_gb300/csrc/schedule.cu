// schedule.cu -- the coarse-to-fine colored ICP schedule for one or many pairs.
//
// reference: color_icp (src/registration/color_icp.hpp:16-63, color_icp.cu:151-234);
// the coarse-to-fine schedule exists in the reference only as a commented example
// (apps/test_color_icp.cpp:378-400).
//
// Per scale, for all pairs at once: voxel-downsample sources and targets (or copy
// them when the scale has no voxel size), build the target grid for normals and
// colour gradients (cell = their largest radius) and, when the correspondence
// distance is smaller, a second, tighter target grid for the NN search; estimate
// target normals and gradients, then launch the two ICP kernels per iteration.  Nothing on the way
// synchronises with the host unless the plain mode is chosen, which, like the
// reference, checks convergence on the host after every iteration.  A plan runs
// the schedule once to size its scratch memory and then captures it as one CUDA
// graph that execute replays; in the graph each scale's iteration loop is a
// conditional WHILE node, so the device stops iterating once every pair converged.
#include "icp.cuh"
#include "stages.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <utility>
#include <vector>

using namespace gca3d;

namespace gca3d
{
int make_segsrc(gca3d_context *ctx, gca3d_cloud *const *clouds, int P, SegSrc **out);
}

struct gca3d_icp_plan
{
    gca3d_context *ctx = nullptr;
    int P = 0;
    std::vector<gca3d_cloud *> src, tgt;
    gca3d_icp_params prm{};
    Arena arena;
    SegSrc *d_src = nullptr, *d_tgt = nullptr;
    PairState *d_state = nullptr;
    PairState *h_state = nullptr;
    double *d_Tinit = nullptr, *h_Tinit = nullptr;
    int max_blocks = 0;
    int max_blocks_nn = 0;
    int64_t src_cap = 0, tgt_cap = 0, src_max = 0, tgt_max = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int64_t kernels_per_run = 0;
    int64_t kernels_static = 0; // graph kernels outside the iteration loops
    bool host_checks = false; // plain mode: convergence test read back after every iteration
    cudaStream_t side = nullptr; // captures the bodies of the device-side loops
    // the preparation branch (every scale's clouds, grids and normals) and its events:
    // the fork after the prologue, and one per scale for the iterations to wait on
    cudaStream_t prep = nullptr;
    cudaEvent_t ev_fork = nullptr;
    cudaEvent_t ev_scale[GCA3D_MAX_SCALES] = {};
    cudaEvent_t ev_grid[GCA3D_MAX_SCALES] = {}; // the scale's search grid is built (before its normals)
    // the source preparation's branch (the first scale's; every scale's in a tracker plan,
    // where the prologue makes the new frame and the target is the previous one)
    cudaStream_t prep_src = nullptr;
    cudaEvent_t ev_fork_src = nullptr;
    cudaEvent_t ev_src[GCA3D_MAX_SCALES] = {};
    int priority = 0; // the device's greatest stream priority (the iterations' kernels)
    PlanPrologue prologue;       // work enqueued before the schedule (captured with it)
    bool vox_given = false;      // voxel batches supplied by the caller
    PlanVoxels vox;
    // the initial poses' copy out of h_Tinit, so that an execute that does not wait for
    // the previous one refills h_Tinit only after that copy has run
    cudaEvent_t tinit_copied = nullptr;
    bool tinit_pending = false;
    // every execute copies the pair states and the device error word back behind the
    // schedule and records states_ready: results() waits for that copy only, so the
    // next execute (of this or another plan) may be queued before the results are read
    cudaEvent_t states_ready = nullptr;
    bool states_pending = false;
    int *h_err = nullptr;
};

namespace
{

int validate_params(gca3d_context *ctx, const gca3d_icp_params *p)
{
    if (!p || p->n_scales < 1 || p->n_scales > GCA3D_MAX_SCALES)
        return fail(ctx, GCA3D_ERR_INVALID_VALUE, "icp: n_scales must be in [1, 8]");
    // cuda_color_icp_build_least_square.cu:438-441
    if (!(p->lambda >= 0.0f && p->lambda <= 1.0f))
        return fail(ctx, GCA3D_ERR_INVALID_VALUE, "icp: lambda must be in [0, 1]");
    if (p->update_map != GCA3D_UPDATE_EULER_ZYX && p->update_map != GCA3D_UPDATE_SE3_EXP)
        return fail(ctx, GCA3D_ERR_INVALID_VALUE, "icp: unknown update map");
    for (int s = 0; s < p->n_scales; ++s)
    {
        const gca3d_scale &S = p->scales[s];
        if (S.max_iter < 0 || !(S.max_corr > 0.0f) || !(S.grad_radius > 0.0f) || S.max_nn < 0 || S.max_nn > 64)
            return fail(ctx, GCA3D_ERR_INVALID_VALUE, "icp: bad scale parameters");
        const bool need_normals = !(S.voxel <= 0.0f && p->keep_target_normals);
        if (need_normals && !(S.normal_radius > 0.0f))
            return fail(ctx, GCA3D_ERR_INVALID_VALUE, "icp: normal radius must be > 0");
    }
    return GCA3D_OK;
}

int read_states(gca3d_icp_plan *pl)
{
    gca3d_context *ctx = pl->ctx;
    GCA_CUDA(ctx, cudaMemcpyAsync(pl->h_state, pl->d_state, sizeof(PairState) * pl->P, cudaMemcpyDeviceToHost,
                                  ctx->stream));
    GCA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return GCA3D_OK;
}

// the scales after si whose voxel sizes halve, exactly in float, one after the other:
// their cells refine scale si's, so one sort at scale si serves them all
SubLevels finer_scales(const gca3d_icp_params &p, int si)
{
    SubLevels sub;
    float v = p.scales[si].voxel;
    for (int k = si + 1; k < p.n_scales && sub.n < kMaxSubLevels; ++k)
    {
        const float w = p.scales[k].voxel;
        if (!(w > 0.0f) || w * 2.0f != v)
            break;
        sub.voxel[sub.n++] = w;
        v = w;
    }
    return sub;
}

// what the iterations of one scale work on, made by the preparation branch
struct ScalePrep
{
    Batch bs, bt;
    Grid gicp; // the grid the correspondence search walks
    float4 *attr0 = nullptr, *attr1 = nullptr;
    double *partials = nullptr;
    int2 *corr = nullptr;
    NNCerts cert{nullptr, nullptr};
    int *bmap = nullptr, *bmap_nn = nullptr;
};

// one scale's clouds, grids, normals, gradients and iteration scratch, enqueued on the
// context stream (the source's on src_stream; grid_ready, if given, recorded once the
// search grid is built); none of it depends on the pose, so it can run ahead of the
// iterations
static int prepare_scale(gca3d_icp_plan *pl, int si, VoxelChain &chain_src, VoxelChain &chain_tgt, ScalePrep &out,
                         cudaStream_t src_stream, cudaEvent_t grid_ready)
{
    gca3d_context *ctx = pl->ctx;
    const gca3d_icp_params &p = pl->prm;
    const int P = pl->P;
    int st = GCA3D_OK;
    const gca3d_scale &S = p.scales[si];
    const bool keep = S.voxel <= 0.0f && p.keep_target_normals;
    Batch &bs = out.bs, &bt = out.bt;
    if (S.voxel > 0.0f)
    {
        // both clouds in Z-order of their voxels: compact source work items, and the
        // same target whether it is downsampled here or supplied
        if (pl->vox_given)
        {
            bs = pl->vox.src[si];
            bt = pl->vox.tgt[si];
        }
        const SubLevels sub = p.tuning.voxel_resort ? SubLevels{} : finer_scales(p, si);
        const bool refine = chain_src.used < chain_src.levels;
        cudaStream_t tgt_stream = ctx->stream;
        ctx->stream = src_stream;
        st = refine ? voxel_refine(ctx, pl->d_src, chain_src, bs)
                    : voxel_stage(ctx, pl->d_src, P, pl->src_cap, pl->src_max, S.voxel, bs, true, &sub, &chain_src);
        ctx->stream = tgt_stream;
        if (st)
            return st;
        if (!pl->vox_given)
        {
            st = chain_tgt.used < chain_tgt.levels
                     ? voxel_refine(ctx, pl->d_tgt, chain_tgt, bt)
                     : voxel_stage(ctx, pl->d_tgt, P, pl->tgt_cap, pl->tgt_max, S.voxel, bt, true, &sub, &chain_tgt);
            if (st)
                return st;
        }
    }
    else
    {
        if ((st = batch_alloc(ctx, bs, P, pl->src_cap, pl->src_max, false, false)))
            return st;
        cudaStream_t tgt_stream = ctx->stream;
        ctx->stream = src_stream;
        st = gather_stage(ctx, pl->d_src, P, pl->src_max, bs, false);
        ctx->stream = tgt_stream;
        if (st)
            return st;
        if ((st = batch_alloc(ctx, bt, P, pl->tgt_cap, pl->tgt_max, keep, false)))
            return st;
        if ((st = gather_stage(ctx, pl->d_tgt, P, pl->tgt_max, bt, keep)))
            return st;
    }
    // the normals / gradient grid (cell = largest of their radii) and, when the
    // correspondence distance is smaller, a tighter grid for the NN search
    float cell_n = S.grad_radius;
    if (!keep)
        cell_n = std::max(cell_n, S.normal_radius);
    const bool own_nn_grid = S.max_corr < 0.9f * cell_n;
    Grid g, gnn;
    if ((st = grid_build(ctx, bt, std::max(cell_n, own_nn_grid ? 0.0f : S.max_corr), kOriginPadF32, nullptr, g)))
        return st;
    if (own_nn_grid && (st = grid_build(ctx, bt, S.max_corr, kOriginPadF32, nullptr, gnn)))
        return st;
    out.gicp = own_nn_grid ? gnn : g;
    if (grid_ready) // the first correspondence search needs the grid, not the normals
        GCA_CUDA(ctx, cudaEventRecord(grid_ready, ctx->stream));
    float4 *attr0 = out.attr0 = ctx->arena.get<float4>(g.cap);
    float4 *attr1 = out.attr1 = ctx->arena.get<float4>(g.cap);
    double *partials = out.partials = ctx->arena.get<double>((size_t)std::max(pl->max_blocks, 1) * kTermsPad);
    int2 *corr = out.corr = ctx->arena.get<int2>(std::max<int64_t>(bs.cap, 1));
    const NNCerts cert = out.cert = NNCerts{ctx->arena.get<float4>(std::max<int64_t>(bs.cap, 1)),
                                            ctx->arena.get<int>(std::max<int64_t>(bs.cap, 1))};
    int *bmap = out.bmap = ctx->arena.get<int>(P + 2); // offsets, total, active pairs
    int *bmap_nn = out.bmap_nn = ctx->arena.get<int>(P + 2); // offsets, total, work queue
    float4 *nrm_b = own_nn_grid && !keep ? ctx->arena.get<float4>(g.cap) : nullptr;
    float4 *grd_b = own_nn_grid ? ctx->arena.get<float4>(g.cap) : nullptr;
    if (!attr0 || !attr1 || !partials || !corr || !cert.pos || !cert.t || !bmap || !bmap_nn || (own_nn_grid && (!grd_b || (!keep && !nrm_b))))
        return fail(ctx, GCA3D_ERR_OUT_OF_MEMORY, "icp: scratch");
    if (own_nn_grid)
    {
        if ((st = normals_stage(ctx, bt, g, !keep, S.normal_radius, S.max_nn, true, S.grad_radius,
                                keep ? bt.nrm : nullptr, nullptr, nullptr, nrm_b, grd_b)))
            return st;
        if ((st = gather_attrs(ctx, bt, gnn, keep ? bt.nrm : nrm_b, grd_b, attr0, attr1)))
            return st;
    }
    else if ((st = normals_stage(ctx, bt, g, !keep, S.normal_radius, S.max_nn, true, S.grad_radius,
                                 keep ? bt.nrm : nullptr, attr0, attr1, nullptr, nullptr)))
        return st;
    return GCA3D_OK;
}

// give every kernel node of a graph the launch priority prio
static cudaError_t prioritise_kernels(cudaGraph_t graph, int prio)
{
    size_t n = 0;
    cudaError_t e = cudaGraphGetNodes(graph, nullptr, &n);
    if (e != cudaSuccess || n == 0)
        return e;
    std::vector<cudaGraphNode_t> nodes(n);
    if ((e = cudaGraphGetNodes(graph, nodes.data(), &n)) != cudaSuccess)
        return e;
    for (cudaGraphNode_t node : nodes)
    {
        cudaGraphNodeType type;
        if ((e = cudaGraphNodeGetType(node, &type)) != cudaSuccess)
            return e;
        if (type != cudaGraphNodeTypeKernel)
            continue;
        cudaKernelNodeAttrValue v = {};
        v.priority = prio;
        if ((e = cudaGraphKernelNodeSetAttribute(node, cudaLaunchAttributePriority, &v)) != cudaSuccess)
            return e;
    }
    return cudaSuccess;
}

// enqueue the whole schedule (eager or under capture): the prologue, the preparation of
// every scale on the plan's preparation stream, forked from the context stream after
// the prologue (with a supplied target, the target's part forked before it and the
// source's on a branch of its own), and the iterations on the context stream, each
// scale's after its preparation; the last scale's events join the streams again
int run_schedule(gca3d_icp_plan *pl, bool capturing)
{
    gca3d_context *ctx = pl->ctx;
    const gca3d_icp_params &p = pl->prm;
    const int P = pl->P;
    cudaStream_t main_stream = ctx->stream;
    // serial: the preparation on the context stream itself (no branch, nothing overlaps).
    // Otherwise the source clouds of the first scale -- and, in a tracker plan, of every
    // scale -- are prepared on a branch of their own beside the target's: nothing else
    // runs before the first scale's iterations, so that preparation is on the critical
    // path.  In a tracker plan the supplied target forks before the prologue.
    const bool serial = p.tuning.serial_prep != 0;
    const bool tracker = !serial && pl->vox_given && pl->prologue;
    cudaStream_t prep = serial ? main_stream : pl->prep;
    cudaStream_t prep_src = serial ? main_stream : pl->prep_src;
    auto src_branch = [&](int si) { return !serial && (tracker || si == 0); };
    int st = GCA3D_OK;
    auto join = [&](int last) {
        // join the branches before giving up (a capture must end on one stream)
        if (serial)
            return;
        cudaEventRecord(pl->ev_fork, prep);
        cudaStreamWaitEvent(main_stream, pl->ev_fork, 0);
        if (last >= 0)
        {
            cudaEventRecord(pl->ev_fork_src, prep_src);
            cudaStreamWaitEvent(main_stream, pl->ev_fork_src, 0);
        }
    };
    if (tracker)
    {
        GCA_CUDA(ctx, cudaEventRecord(pl->ev_fork, main_stream));
        GCA_CUDA(ctx, cudaStreamWaitEvent(prep, pl->ev_fork, 0));
    }
    if (pl->prologue && (st = pl->prologue(ctx)))
    {
        if (tracker)
            join(-1);
        return st;
    }
    if ((st = icp_state_init(ctx, pl->d_state, P, pl->d_Tinit)))
    {
        if (tracker)
            join(-1);
        return st;
    }
    if (!serial)
    {
        GCA_CUDA(ctx, cudaEventRecord(pl->ev_fork_src, main_stream));
        GCA_CUDA(ctx, cudaStreamWaitEvent(prep_src, pl->ev_fork_src, 0));
        if (!tracker)
            GCA_CUDA(ctx, cudaStreamWaitEvent(prep, pl->ev_fork_src, 0));
    }
    ScalePrep sp[GCA3D_MAX_SCALES];
    {
        VoxelChain chain_src, chain_tgt; // sorted state of the last voxel stage, for finer scales
        ctx->stream = prep;
        for (int si = 0; si < p.n_scales && !st; ++si)
        {
            // a finer scale's source continues the first scale's sorted state
            if (!serial && !tracker && si == 1)
            {
                const cudaError_t e = cudaStreamWaitEvent(prep, pl->ev_src[0], 0);
                if (e != cudaSuccess)
                {
                    st = cuda_fail(ctx, e, "icp: preparation event");
                    break;
                }
            }
            st = prepare_scale(pl, si, chain_src, chain_tgt, sp[si], src_branch(si) ? prep_src : prep,
                               serial ? nullptr : pl->ev_grid[si]);
            if (!st && !serial)
            {
                cudaError_t e = cudaEventRecord(pl->ev_scale[si], prep);
                if (e == cudaSuccess && src_branch(si))
                    e = cudaEventRecord(pl->ev_src[si], prep_src);
                if (e != cudaSuccess)
                    st = cuda_fail(ctx, e, "icp: preparation event");
            }
        }
        ctx->stream = main_stream;
        if (st)
        {
            join(0);
            return st;
        }
    }
    // the iterations, each scale's after its preparation
    auto iterate = [&]() -> int {
        for (int si = 0; si < p.n_scales; ++si)
        {
            const gca3d_scale &S = p.scales[si];
            // the first search waits for the clouds and the search grid, the iterations
            // for the normals and gradients too
            if (!serial)
                GCA_CUDA(ctx, cudaStreamWaitEvent(main_stream, pl->ev_grid[si], 0));
            if (src_branch(si))
                GCA_CUDA(ctx, cudaStreamWaitEvent(main_stream, pl->ev_src[si], 0));
            const Batch &bs = sp[si].bs, &bt = sp[si].bt;
            const Grid &gicp = sp[si].gicp;
            float4 *attr0 = sp[si].attr0, *attr1 = sp[si].attr1;
            double *partials = sp[si].partials;
            int2 *corr = sp[si].corr;
            const NNCerts cert = sp[si].cert;
            int *bmap = sp[si].bmap, *bmap_nn = sp[si].bmap_nn;
            const IcpShape shape = icp_shape(p.tuning);
            if ((st = icp_setup(ctx, pl->d_state, P, bs.seg_off, bt.seg_off, bmap, bmap_nn, si, shape.nn_chunk)))
                return st;
            IcpScale prm;
            prm.max_corr = S.max_corr;
            prm.sqrt_lg = sqrtf(p.lambda);
            prm.sqrt_lc = sqrtf(1.0f - p.lambda);
            prm.update_map = p.update_map;
            prm.rot_eps = p.rot_eps;
            prm.trans_eps = p.trans_eps;
            // loop counter and finalize ticket
            int *iter = ctx->arena.get<int>(2);
            if (!iter)
                return fail(ctx, GCA3D_ERR_OUT_OF_MEMORY, "icp: scratch");
            GCA_CUDA(ctx, cudaMemsetAsync(iter, 0, 2 * sizeof(int), ctx->stream));
            IcpLoop loop;
            loop.ticket = reinterpret_cast<unsigned *>(iter + 1);
            if (S.max_iter > 0 &&
                (st = icp_search(ctx, bs, gicp, pl->d_state, bmap_nn, pl->max_blocks_nn, corr, cert, prm, nullptr,
                                 nullptr, shape)))
                return st;
            if (!serial)
                GCA_CUDA(ctx, cudaStreamWaitEvent(main_stream, pl->ev_scale[si], 0));
            if (capturing && S.max_iter > 0)
            {
                // the iteration loop as a device-side WHILE node: the body runs while a
                // pair is active and the budget lasts, so converged schedules stop early
                cudaStreamCaptureStatus cs;
                cudaGraph_t cg = nullptr;
                const cudaGraphNode_t *deps = nullptr;
                size_t nd = 0;
                GCA_CUDA(ctx, cudaStreamGetCaptureInfo(ctx->stream, &cs, nullptr, &cg, &deps, nullptr, &nd));
                cudaGraphConditionalHandle handle;
                GCA_CUDA(ctx, cudaGraphConditionalHandleCreate(&handle, cg, 1, cudaGraphCondAssignDefault));
                cudaGraphNodeParams np = {};
                np.type = cudaGraphNodeTypeConditional;
                np.conditional.handle = handle;
                np.conditional.type = cudaGraphCondTypeWhile;
                np.conditional.size = 1;
                cudaGraphNode_t node;
                GCA_CUDA(ctx, cudaGraphAddNode(&node, cg, deps, nullptr, nd, &np));
                cudaGraph_t body = np.conditional.phGraph_out[0];
                GCA_CUDA(ctx, cudaStreamBeginCaptureToGraph(pl->side, body, nullptr, nullptr, 0,
                                                            cudaStreamCaptureModeThreadLocal));
                ctx->stream = pl->side;
                const int64_t l0 = ctx->launches;
                loop.handle = handle;
                loop.iter = iter;
                loop.max_iter = S.max_iter;
                // the body: this iteration's update, then the next iteration's search
                // (which returns at once once the budget is spent)
                st = icp_update(ctx, bs, gicp, attr0, attr1, pl->d_state, bmap, pl->max_blocks, bmap_nn, partials,
                                corr, prm, p.compensated != 0, loop, shape);
                if (!st)
                    st = icp_search(ctx, bs, gicp, pl->d_state, bmap_nn, pl->max_blocks_nn, corr, cert, prm,
                                    nullptr, &loop, shape);
                pl->kernels_static -= ctx->launches - l0; // counted per iteration instead
                ctx->stream = main_stream;
                cudaGraph_t captured = nullptr;
                const cudaError_t e = cudaStreamEndCapture(pl->side, &captured);
                if (st)
                    return st;
                GCA_CUDA(ctx, e);
                // the iterations are the critical path: their kernels go first where the
                // preparation branch's kernels compete for the same SMs
                GCA_CUDA(ctx, prioritise_kernels(body, pl->priority));
                GCA_CUDA(ctx, cudaStreamUpdateCaptureDependencies(ctx->stream, &node, nullptr, 1,
                                                                  cudaStreamSetCaptureDependencies));
                continue;
            }
            for (int it = 0; it < S.max_iter; ++it)
            {
                if ((st = icp_update(ctx, bs, gicp, attr0, attr1, pl->d_state, bmap, pl->max_blocks, bmap_nn,
                                     partials, corr, prm, p.compensated != 0, loop, shape)))
                    return st;
                if (pl->host_checks && !capturing)
                {
                    // the reference's control flow: the step is inspected on the host
                    if ((st = read_states(pl)))
                        return st;
                    bool any = false;
                    for (int k = 0; k < P; ++k)
                        any |= pl->h_state[k].active != 0;
                    if (!any)
                        break;
                }
                if (it + 1 < S.max_iter &&
                    (st = icp_search(ctx, bs, gicp, pl->d_state, bmap_nn, pl->max_blocks_nn, corr, cert, prm,
                                     nullptr, nullptr, shape)))
                    return st;
            }
        }

        return GCA3D_OK;
    };
    st = iterate();
    if (st && !serial) // join the branches before giving up
    {
        cudaStreamWaitEvent(main_stream, pl->ev_scale[p.n_scales - 1], 0);
        cudaStreamWaitEvent(main_stream, pl->ev_src[tracker ? p.n_scales - 1 : 0], 0);
    }
    return st;
}

int run_with_arena(gca3d_icp_plan *pl, bool capturing)
{
    pl->ctx->arena.swap(pl->arena);
    pl->ctx->arena.reset();
    const int64_t l0 = pl->ctx->launches;
    pl->kernels_static = 0;
    int st = run_schedule(pl, capturing);
    if (!st && pl->ctx->arena.failed)
        st = fail(pl->ctx, GCA3D_ERR_OUT_OF_MEMORY, "icp plan: scratch memory");
    pl->kernels_per_run = pl->ctx->launches - l0;
    if (capturing)
        pl->kernels_static += pl->kernels_per_run;
    pl->ctx->arena.swap(pl->arena);
    return st;
}

void fill_results(const gca3d_icp_plan *pl, gca3d_icp_result *res)
{
    for (int k = 0; k < pl->P; ++k)
    {
        const PairState &S = pl->h_state[k];
        gca3d_icp_result &r = res[k];
        memcpy(r.T, S.T, sizeof r.T);
        r.rmse_ref = S.rmse_ref;
        r.fitness = S.fitness;
        r.inlier_rmse = S.inlier_rmse;
        r.iterations = S.iters;
        r.converged = S.converged;
        r.status = S.status;
        r.n_src = S.nsrc;
        r.n_tgt = S.ntgt;
        for (int k = 0; k < GCA3D_MAX_SCALES; ++k)
        {
            r.scale_iterations[k] = S.scale_iters[k];
            r.scale_n_src[k] = S.scale_nsrc[k];
            r.scale_n_tgt[k] = S.scale_ntgt[k];
        }
    }
}

} // namespace

extern "C" {

int gca3d_icp_plan_destroy(gca3d_icp_plan *pl)
{
    if (!pl)
        return GCA3D_ERR_INVALID_VALUE;
    if (pl->ctx)
        cudaStreamSynchronize(pl->ctx->stream);
    if (pl->exec)
        cudaGraphExecDestroy(pl->exec);
    if (pl->tinit_copied)
        cudaEventDestroy(pl->tinit_copied);
    if (pl->states_ready)
        cudaEventDestroy(pl->states_ready);
    if (pl->h_err)
        cudaFreeHost(pl->h_err);
    if (pl->side)
        cudaStreamDestroy(pl->side);
    if (pl->prep)
        cudaStreamDestroy(pl->prep);
    if (pl->prep_src)
        cudaStreamDestroy(pl->prep_src);
    if (pl->ev_fork_src)
        cudaEventDestroy(pl->ev_fork_src);
    for (cudaEvent_t e : pl->ev_src)
        if (e)
            cudaEventDestroy(e);
    for (cudaEvent_t e : pl->ev_grid)
        if (e)
            cudaEventDestroy(e);
    if (pl->ev_fork)
        cudaEventDestroy(pl->ev_fork);
    for (cudaEvent_t e : pl->ev_scale)
        if (e)
            cudaEventDestroy(e);
    if (pl->graph)
        cudaGraphDestroy(pl->graph);
    cudaFree(pl->d_src);
    cudaFree(pl->d_tgt);
    cudaFree(pl->d_state);
    cudaFree(pl->d_Tinit);
    if (pl->h_state)
        cudaFreeHost(pl->h_state);
    if (pl->h_Tinit)
        cudaFreeHost(pl->h_Tinit);
    pl->arena.release();
    delete pl;
    return GCA3D_OK;
}

} // extern "C"

int gca3d::icp_plan_create_internal(gca3d_context *ctx, int P, gca3d_cloud *const *src, gca3d_cloud *const *tgt,
                                    const gca3d_icp_params *params, bool capture, PlanPrologue prologue,
                                    gca3d_icp_plan **out, const PlanVoxels *voxels)
{
    if (!ctx || !out || P < 1 || P > kMaxSegments || !src || !tgt)
        return fail(ctx, GCA3D_ERR_INVALID_VALUE, "icp: bad arguments (1 <= pairs <= 4096)");
    *out = nullptr;
    int st = validate_params(ctx, params);
    if (st)
        return st;
    for (int k = 0; k < P; ++k)
    {
        if (!src[k] || !tgt[k])
            return fail(ctx, GCA3D_ERR_INVALID_VALUE, "icp: null cloud");
        if (params->keep_target_normals && params->scales[0].voxel <= 0.0f && !tgt[k]->has_normals)
            return fail(ctx, GCA3D_ERR_INVALID_VALUE, "icp: the target has no normals (estimate normals first)");
    }
    auto *pl = new gca3d_icp_plan();
    pl->ctx = ctx;
    pl->P = P;
    pl->src.assign(src, src + P);
    pl->tgt.assign(tgt, tgt + P);
    pl->prm = *params;
    pl->host_checks = !params->use_graph;
    pl->prologue = std::move(prologue);
    if (voxels)
    {
        for (int s = 0; s < params->n_scales; ++s)
            if (!(params->scales[s].voxel > 0.0f))
            {
                delete pl;
                return fail(ctx, GCA3D_ERR_INVALID_VALUE, "icp: supplied voxel batches need a voxel size at every scale");
            }
        if (P != 1)
        {
            delete pl;
            return fail(ctx, GCA3D_ERR_INVALID_VALUE, "icp: supplied voxel batches are for one pair");
        }
        pl->vox_given = true;
        pl->vox = *voxels;
    }
    int nb = 0;
    for (int k = 0; k < P; ++k)
    {
        pl->src_cap += src[k]->capacity;
        pl->tgt_cap += tgt[k]->capacity;
        pl->src_max = std::max(pl->src_max, src[k]->capacity);
        pl->tgt_max = std::max(pl->tgt_max, tgt[k]->capacity);
        nb += div_up(src[k]->capacity, kIcpChunk);
        pl->max_blocks_nn += div_up(src[k]->capacity, icp_shape(params->tuning).nn_chunk);
    }
    pl->max_blocks = std::max(nb, 1);
    pl->max_blocks_nn = std::max(pl->max_blocks_nn, 1);
    // device tables and state live outside the scratch arena
    std::vector<SegSrc> hs(P), ht(P);
    for (int k = 0; k < P; ++k)
    {
        hs[k] = SegSrc{src[k]->pos, src[k]->col, nullptr, src[k]->d_count};
        ht[k] = SegSrc{tgt[k]->pos, tgt[k]->col, tgt[k]->has_normals ? tgt[k]->nrm : nullptr, tgt[k]->d_count};
    }
    if (cudaMalloc(&pl->d_src, sizeof(SegSrc) * P) != cudaSuccess ||
        cudaMalloc(&pl->d_tgt, sizeof(SegSrc) * P) != cudaSuccess ||
        cudaMalloc(&pl->d_state, sizeof(PairState) * P) != cudaSuccess ||
        cudaMalloc(&pl->d_Tinit, sizeof(double) * 16 * P) != cudaSuccess ||
        cudaMallocHost(&pl->h_state, sizeof(PairState) * P) != cudaSuccess ||
        cudaMallocHost(&pl->h_err, sizeof(int)) != cudaSuccess ||
        cudaMallocHost(&pl->h_Tinit, sizeof(double) * 16 * P) != cudaSuccess)
    {
        cudaGetLastError();
        gca3d_icp_plan_destroy(pl);
        return fail(ctx, GCA3D_ERR_OUT_OF_MEMORY, "icp plan: allocation");
    }
    cudaMemcpy(pl->d_src, hs.data(), sizeof(SegSrc) * P, cudaMemcpyHostToDevice);
    cudaMemcpy(pl->d_tgt, ht.data(), sizeof(SegSrc) * P, cudaMemcpyHostToDevice);
    for (int k = 0; k < P; ++k)
        for (int j = 0; j < 16; ++j)
            pl->h_Tinit[16 * k + j] = (j % 5 == 0) ? 1.0 : 0.0;
    cudaMemcpy(pl->d_Tinit, pl->h_Tinit, sizeof(double) * 16 * P, cudaMemcpyHostToDevice);
    if (capture && cudaStreamCreateWithFlags(&pl->side, cudaStreamNonBlocking) != cudaSuccess)
    {
        cudaGetLastError();
        gca3d_icp_plan_destroy(pl);
        return fail(ctx, GCA3D_ERR_CUDA, "icp plan: side stream");
    }
    int least_prio = 0;
    if (cudaDeviceGetStreamPriorityRange(&least_prio, &pl->priority) != cudaSuccess)
        pl->priority = 0;
    bool events_ok = cudaStreamCreateWithFlags(&pl->prep, cudaStreamNonBlocking) == cudaSuccess &&
                     cudaEventCreateWithFlags(&pl->ev_fork, cudaEventDisableTiming) == cudaSuccess;
    for (int k = 0; k < params->n_scales && events_ok; ++k)
        events_ok = cudaEventCreateWithFlags(&pl->ev_scale[k], cudaEventDisableTiming) == cudaSuccess &&
                    cudaEventCreateWithFlags(&pl->ev_grid[k], cudaEventDisableTiming) == cudaSuccess;
    if (events_ok)
    {
        events_ok = cudaStreamCreateWithFlags(&pl->prep_src, cudaStreamNonBlocking) == cudaSuccess &&
                    cudaEventCreateWithFlags(&pl->ev_fork_src, cudaEventDisableTiming) == cudaSuccess;
        for (int k = 0; k < params->n_scales && events_ok; ++k)
            events_ok = cudaEventCreateWithFlags(&pl->ev_src[k], cudaEventDisableTiming) == cudaSuccess;
    }
    if (!events_ok)
    {
        cudaGetLastError();
        gca3d_icp_plan_destroy(pl);
        return fail(ctx, GCA3D_ERR_CUDA, "icp plan: preparation stream");
    }
    if (capture)
    {
        // size the scratch with one eager run, then capture the identical sequence
        st = run_with_arena(pl, false);
        if (!st)
        {
            cudaError_t e = cudaStreamSynchronize(ctx->stream);
            st = e != cudaSuccess ? cuda_fail(ctx, e, "icp plan warm-up") : consume_device_error(ctx, "icp plan");
        }
        if (!st)
        {
            pl->arena.frozen = true;
            cudaError_t e = cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal);
            if (e != cudaSuccess)
                st = cuda_fail(ctx, e, "cudaStreamBeginCapture");
            else
            {
                int st2 = run_with_arena(pl, true);
                cudaGraph_t g = nullptr;
                e = cudaStreamEndCapture(ctx->stream, &g);
                pl->graph = g;
                if (st2)
                    st = st2;
                else if (e != cudaSuccess)
                    st = cuda_fail(ctx, e, "cudaStreamEndCapture");
                else
                {
                    e = cudaGraphInstantiate(&pl->exec, pl->graph, cudaGraphInstantiateFlagUseNodePriority);
                    if (e != cudaSuccess)
                        st = cuda_fail(ctx, e, "cudaGraphInstantiate");
                    // until an execute reports iteration counts: every loop runs to its budget
                    int64_t budget = 0;
                    for (int s = 0; s < params->n_scales; ++s)
                        budget += params->scales[s].max_iter;
                    pl->kernels_per_run = pl->kernels_static + 3 * budget;
                }
            }
            pl->arena.frozen = false;
        }
        if (st)
        {
            cudaGetLastError();
            gca3d_icp_plan_destroy(pl);
            return st;
        }
    }
    *out = pl;
    return GCA3D_OK;
}

extern "C" {

int gca3d_icp_plan_create(gca3d_context *ctx, int n_pairs, gca3d_cloud *const *src, gca3d_cloud *const *tgt,
                          const gca3d_icp_params *params, gca3d_icp_plan **plan)
{
    return icp_plan_create_internal(ctx, n_pairs, src, tgt, params, params && params->use_graph, nullptr, plan);
}

int gca3d_icp_plan_execute(gca3d_icp_plan *pl, const double *T_init, gca3d_icp_result *results)
{
    if (!pl)
        return GCA3D_ERR_INVALID_VALUE;
    gca3d_context *ctx = pl->ctx;
    if (!pl->tinit_copied)
        GCA_CUDA(ctx, cudaEventCreateWithFlags(&pl->tinit_copied, cudaEventDisableTiming));
    if (pl->tinit_pending)
        GCA_CUDA(ctx, cudaEventSynchronize(pl->tinit_copied));
    for (int k = 0; k < pl->P; ++k)
        for (int j = 0; j < 16; ++j)
            pl->h_Tinit[16 * k + j] = T_init ? T_init[16 * k + j] : ((j % 5 == 0) ? 1.0 : 0.0);
    GCA_CUDA(ctx, cudaMemcpyAsync(pl->d_Tinit, pl->h_Tinit, sizeof(double) * 16 * pl->P, cudaMemcpyHostToDevice,
                                  ctx->stream));
    GCA_CUDA(ctx, cudaEventRecord(pl->tinit_copied, ctx->stream));
    pl->tinit_pending = true;
    int st;
    if (pl->exec)
    {
        GCA_CUDA(ctx, cudaGraphLaunch(pl->exec, ctx->stream));
        if (!results) // iteration counts unknown: the previous execute's count stands in
            ctx->launches += pl->kernels_per_run;
    }
    else if ((st = run_with_arena(pl, false)))
        return st;
    if (!pl->states_ready)
        GCA_CUDA(ctx, cudaEventCreateWithFlags(&pl->states_ready, cudaEventDisableTiming));
    GCA_CUDA(ctx, cudaMemcpyAsync(pl->h_state, pl->d_state, sizeof(PairState) * pl->P, cudaMemcpyDeviceToHost,
                                  ctx->stream));
    GCA_CUDA(ctx, cudaMemcpyAsync(pl->h_err, ctx->d_err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    GCA_CUDA(ctx, cudaMemsetAsync(ctx->d_err, 0, sizeof(int), ctx->stream));
    GCA_CUDA(ctx, cudaEventRecord(pl->states_ready, ctx->stream));
    pl->states_pending = true;
    if (!results)
        return GCA3D_OK;
    return gca3d_icp_plan_results(pl, results);
}

int gca3d_icp_plan_results(gca3d_icp_plan *pl, gca3d_icp_result *results)
{
    if (!pl || !results)
        return GCA3D_ERR_INVALID_VALUE;
    gca3d_context *ctx = pl->ctx;
    if (!pl->states_pending)
        return fail(ctx, GCA3D_ERR_INVALID_VALUE, "icp: results of a plan never executed");
    GCA_CUDA(ctx, cudaEventSynchronize(pl->states_ready));
    int st;
    if ((st = device_error_status(ctx, *pl->h_err, "icp")))
        return st;
    fill_results(pl, results);
    if (pl->exec)
    {
        int64_t loops = 0;
        for (int s = 0; s < pl->prm.n_scales; ++s)
        {
            int m = 0;
            for (int k = 0; k < pl->P; ++k)
                m = std::max(m, pl->h_state[k].scale_iters[s]);
            loops += pl->prm.scales[s].max_iter > 0 ? std::max(m, 1) : 0;
        }
        pl->kernels_per_run = pl->kernels_static + 3 * loops;
        ctx->launches += pl->kernels_per_run;
    }
    return GCA3D_OK;
}

int gca3d_icp_plan_readback_bytes(gca3d_icp_plan *pl, int64_t *bytes)
{
    if (!pl || !bytes)
        return GCA3D_ERR_INVALID_VALUE;
    *bytes = (int64_t)sizeof(PairState) * pl->P + (int64_t)sizeof(int);
    return GCA3D_OK;
}

int gca3d_icp_plan_kernels(gca3d_icp_plan *pl, int64_t *n)
{
    if (!pl || !n)
        return GCA3D_ERR_INVALID_VALUE;
    *n = pl->kernels_per_run;
    return GCA3D_OK;
}

int gca3d_color_icp_batched(gca3d_context *ctx, int n_pairs, gca3d_cloud *const *src, gca3d_cloud *const *tgt,
                            const gca3d_icp_params *params, const double *T_init, gca3d_icp_result *results)
{
    if (!results)
        return fail(ctx, GCA3D_ERR_INVALID_VALUE, "icp: results needed");
    gca3d_icp_plan *pl = nullptr;
    int st = icp_plan_create_internal(ctx, n_pairs, src, tgt, params, false, nullptr, &pl);
    if (st)
        return st;
    st = gca3d_icp_plan_execute(pl, T_init, results);
    gca3d_icp_plan_destroy(pl);
    return st;
}

int gca3d_color_icp(gca3d_context *ctx, gca3d_cloud *src, gca3d_cloud *tgt, const gca3d_icp_params *params,
                    const double T_init[16], gca3d_icp_result *result)
{
    return gca3d_color_icp_batched(ctx, 1, &src, &tgt, params, T_init, result);
}

} // extern "C"

// ---------------------------------------------------------------------------
// launch-shape autotuner: coordinate descent over the launch-shape knobs of
// gca3d_tuning (item size, the two grids, the finalize's own launch or not), each
// candidate timed on the caller's workload as a fresh plan (one warm-up execute,
// then `reps` executes between CUDA events on the context stream)
// ---------------------------------------------------------------------------
extern "C" int gca3d_icp_autotune(gca3d_context *ctx, int n_pairs, gca3d_cloud *const *src, gca3d_cloud *const *tgt,
                                  const gca3d_icp_params *params, int reps, gca3d_tuning *best, double *best_ms)
{
    if (!ctx || !params || !src || !tgt || n_pairs < 1)
        return fail(ctx, GCA3D_ERR_INVALID_VALUE, "autotune: bad arguments");
    reps = std::max(reps, 1);
    gca3d_icp_params p = *params;
    const IcpShape s0 = icp_shape(p.tuning);
    gca3d_tuning cur{s0.nn_chunk, s0.nn_bps, s0.acc_bps, p.tuning.voxel_resort, s0.fused ? 1 : 0,
                     p.tuning.serial_prep};
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)
    {
        cudaGetLastError();
        if (e0)
            cudaEventDestroy(e0);
        return fail(ctx, GCA3D_ERR_CUDA, "autotune: events");
    }
    auto time_one = [&](const gca3d_tuning &t, double &ms) -> int {
        p.tuning = t;
        gca3d_icp_plan *pl = nullptr;
        int st = icp_plan_create_internal(ctx, n_pairs, src, tgt, &p, p.use_graph != 0, nullptr, &pl);
        if (st)
            return st;
        st = gca3d_icp_plan_execute(pl, nullptr, nullptr);
        if (!st && cudaEventRecord(e0, ctx->stream) != cudaSuccess)
            st = cuda_fail(ctx, cudaGetLastError(), "autotune: event");
        for (int r = 0; r < reps && !st; ++r)
            st = gca3d_icp_plan_execute(pl, nullptr, nullptr);
        if (!st)
        {
            cudaError_t e = cudaEventRecord(e1, ctx->stream);
            if (e == cudaSuccess)
                e = cudaEventSynchronize(e1);
            float f = 0.0f;
            if (e == cudaSuccess)
                e = cudaEventElapsedTime(&f, e0, e1);
            if (e != cudaSuccess)
                st = cuda_fail(ctx, e, "autotune: timing");
            ms = (double)f / reps;
        }
        gca3d_icp_plan_destroy(pl);
        if (!st)
            st = consume_device_error(ctx, "autotune");
        return st;
    };
    double best_t = 0.0;
    int st = time_one(cur, best_t);
    const int nn_items[] = {64, 128, 256, 512};
    const int nn_bps[] = {4, 6, 8, 10, 14, 20};
    const int acc_bps[] = {2, 3, 4, 6, 8, 12};
    const int fused[] = {0, 1};
    for (int knob = 0; knob < 4 && !st; ++knob)
    {
        const int *vals = knob == 0 ? nn_items : (knob == 1 ? nn_bps : (knob == 2 ? acc_bps : fused));
        const int nv = knob == 0 ? 4 : (knob == 3 ? 2 : 6);
        for (int v = 0; v < nv && !st; ++v)
        {
            gca3d_tuning t = cur;
            int &field = knob == 0 ? t.nn_item_points
                                   : (knob == 1 ? t.nn_blocks_per_sm
                                                : (knob == 2 ? t.accum_blocks_per_sm : t.fused_finalize));
            if (field == vals[v])
                continue;
            field = vals[v];
            double ms = 0.0;
            st = time_one(t, ms);
            if (!st && ms < best_t)
            {
                best_t = ms;
                cur = t;
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (st)
        return st;
    if (best)
        *best = cur;
    if (best_ms)
        *best_ms = best_t;
    return GCA3D_OK;
}
