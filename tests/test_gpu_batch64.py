"""The throughput workload (64 fragment pairs) against the FP64 oracle.

Clouds of 20k-300k points (log-uniform), per-pair rotation 0-15 deg and
translation 0-15 cm, overlap 40-90 %, three scales (voxel 0.04 / 0.02 / 0.01 m,
50 / 30 / 14 iterations, SE(3) steps).  Both GPU arms -- the batched graph plan
with compensated accumulation, and the FP32 path that registers one pair per call
with eager launches -- must stop after the same number of iterations at every
scale as the FP64 oracle and end within 1e-5 rad and 1e-5 m of its pose, on every
pair.  One pair of the batch (index 50) converges to a wrong local minimum 0.12
rad from the ground truth; the oracle does the same, and the bar holds there too."""
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
    orc.set_threads(os.cpu_count() or 1)
    try:
        out = []
        for p in batch:
            T, res = orc.multiscale_f64(p.src_xyz, p.src_rgb, p.tgt_xyz, p.tgt_rgb, [orc.Scale(*s) for s in SCALES],
                                        update_map=orc.UPDATE_SE3_EXP)
            out.append((T, [r.iterations for r in res]))
        return out
    finally:
        orc.set_threads(1)


def check_arm(name, results, oracle_runs, synth, batch):
    errs = np.array([synth.pose_error(r["T"], T64) for r, (T64, _) in zip(results, oracle_runs)])
    its = [(i, r["scale_iterations"][:3], it) for i, (r, (_, it)) in enumerate(zip(results, oracle_runs))
           if list(r["scale_iterations"][:3]) != it]
    assert not its, f"{name}: per-scale iterations differ from the oracle (pair, gpu, oracle): {its}"
    worst = np.argsort(-errs.max(1))[:3]
    msg = f"{name}: worst pairs " + ", ".join(f"{i}: {errs[i, 0]:.2e} rad {errs[i, 1]:.2e} m" for i in worst)
    assert errs[:, 0].max() <= POSE_TOL and errs[:, 1].max() <= POSE_TOL, msg
    return errs


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
    gt = [synth.pose_error(T64, p.T_gt)[0] for (T64, _), p in zip(oracle_runs, batch)]
    assert int(np.argmax(gt)) == 50 and gt[50] > 0.1
