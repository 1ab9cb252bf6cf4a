"""The throughput workload (64 fragment pairs) against the FP64 oracle.

Clouds of 20k-300k points (log-uniform), per-pair rotation 0-15 deg and
translation 0-15 cm, overlap 40-90 %, three scales (voxel 0.04 / 0.02 / 0.01 m,
50 / 30 / 14 iterations, SE(3) steps).  Both GPU arms -- the batched graph plan
with compensated accumulation, and the FP32 path that registers one pair per call
with eager launches -- must stop after the same number of iterations at every
scale as the FP64 oracle and end within 1e-5 rad and 1e-5 m of its pose, on every
pair.  The oracle runs in two modes: correspondences searched on FP64 points, and
on the FP32 points the GPU searches (pose rounded to float, fused application,
FP32 squared distances; everything else FP64).  The two agree within 1e-5 except at
a pair whose correspondences sit on a bifurcation (pair 13: 3.4e-6 rad, 2.2e-5 m
apart); there an FP32 rounding anywhere may tip the GPU to either side, so a pair
passes when it is within the bar of either mode (with that mode's iteration counts).
One pair (index 50) converges to a wrong local minimum 0.12 rad from the ground
truth; the oracle does the same, and the bar holds there too."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

POSE_TOL = 1e-5
SCALES = [(0.04, 50, 0.06, 0.08, 0.08), (0.02, 30, 0.03, 0.04, 0.04), (0.01, 14, 0.015, 0.02, 0.02)]


@pytest.fixture(scope="module")
def N():
    from cuda_3d_gb300 import build, native

    build.build()
    return native


@pytest.fixture(scope="module")
def ctx(N):
    return N.Context(0)


@pytest.fixture(scope="module")
def synth():
    from cuda_3d_gb300 import synth as S

    return S


@pytest.fixture(scope="module")
def batch(synth):
    return synth.batch_pairs(64, seed=0, sampler=synth.RoomSampler())


@pytest.fixture(scope="module")
def oracle_runs(orc, batch):
    """per pair: {search mode: (pose, per-scale iterations)} for the FP64 and FP32 searches"""
    orc.set_threads(os.cpu_count() or 1)
    try:
        out = []
        for p in batch:
            runs = {}
            for mode in ("fp64", "fp32"):
                T, res = orc.multiscale_f64(p.src_xyz, p.src_rgb, p.tgt_xyz, p.tgt_rgb,
                                            [orc.Scale(*s) for s in SCALES], update_map=orc.UPDATE_SE3_EXP,
                                            search_f32=mode == "fp32")
                runs[mode] = (T, [r.iterations for r in res])
            out.append(runs)
        return out
    finally:
        orc.set_threads(1)


def check_arm(name, results, oracle_runs, synth, batch):
    bad = []
    for i, (r, runs) in enumerate(zip(results, oracle_runs)):
        fits = {}
        for mode, (T64, it) in runs.items():
            rot, tr = synth.pose_error(r["T"], T64)
            fits[mode] = (rot, tr, list(r["scale_iterations"][:3]) == it)
        if not any(rot <= POSE_TOL and tr <= POSE_TOL and same for rot, tr, same in fits.values()):
            bad.append((i, {m: f"{v[0]:.2e} rad {v[1]:.2e} m, iterations equal: {v[2]}" for m, v in fits.items()}))
    assert not bad, f"{name}: pairs outside the bar of both oracle modes: {bad}"
    # the strict FP64 mode alone holds everywhere but at bifurcation pairs, where the two
    # oracle modes are themselves further apart than the bar
    for i, (r, runs) in enumerate(zip(results, oracle_runs)):
        rot, tr = synth.pose_error(r["T"], runs["fp64"][0])
        if rot > POSE_TOL or tr > POSE_TOL:
            orot, otr = synth.pose_error(runs["fp64"][0], runs["fp32"][0])
            assert orot > POSE_TOL or otr > POSE_TOL, (name, i, rot, tr)


def test_batch64_both_arms_match_fp64_oracle(ctx, N, synth, batch, oracle_runs):
    srcs = [ctx.cloud_from(p.src_xyz, p.src_rgb) for p in batch]
    tgts = [ctx.cloud_from(p.tgt_xyz, p.tgt_rgb) for p in batch]
    scales = [N.scale(*s) for s in SCALES]
    chosen = N.IcpPlan(ctx, srcs, tgts, N.icp_params(scales, update_map=N.UPDATE_SE3_EXP, compensated=True,
                                                      use_graph=True)).execute(results=True)
    pp = N.icp_params(scales, update_map=N.UPDATE_SE3_EXP, compensated=False, use_graph=False)
    plain = [N.color_icp(ctx, s, t, pp) for s, t in zip(srcs, tgts)]
    check_arm("chosen", chosen, oracle_runs, synth, batch)
    check_arm("plain", plain, oracle_runs, synth, batch)
    # the wrong local minimum is the algorithm's, not the GPU's
    gt = [synth.pose_error(runs["fp64"][0], p.T_gt)[0] for runs, p in zip(oracle_runs, batch)]
    assert int(np.argmax(gt)) == 50 and gt[50] > 0.1
