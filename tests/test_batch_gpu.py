"""Batched uneven wave instances: per-instance parity with the FP64 oracle,
CUDA-graph replay, and the autotuned persistent launch."""
import numpy as np
import pytest
import torch

from oracle import wave as W

pytestmark = pytest.mark.gpu


def _oracle(inst):
    s = W.WaveSetup(inst["nt"], inst["nx"], inst["init_u"], inst["init_ut"],
                    inst["left_u"], inst["right_u"], c=inst["c"])
    return W.solve_march(s, rounds=2)


def _small_batch():
    from odil_gb300.workloads import wave_batch_instances
    return wave_batch_instances(count=24, seed=9, nmin=5, nmax=70)


def test_batch_matches_oracle_per_instance(cuda):
    from odil_gb300.batch import WaveBatch
    insts = _small_batch()
    assert len({i["nx"] % 4 for i in insts}) > 1  # vector and scalar paths
    b = WaveBatch(insts, device=cuda)
    b.solve_mixed(epochs=2)
    got = b.unpack()
    for inst, u in zip(insts, got):
        ref = _oracle(inst)
        assert W.rel_err(u, ref) <= 1e-8, (inst["nt"], inst["c"])


def test_graph_replay_and_autotune(cuda, tmp_path, monkeypatch):
    monkeypatch.setenv("ODIL_GB300_TUNE_CACHE", str(tmp_path / "tune.json"))
    from odil_gb300.batch import WaveBatch
    from odil_gb300 import autotune
    insts = _small_batch()
    b = WaveBatch(insts, device=cuda)
    cfg = b.tune()
    assert cfg in autotune.candidates_batch_march(b.max_nx)
    assert (tmp_path / "tune.json").exists()
    b.solve_mixed()
    eager = b.u.clone()
    b.capture()
    b.u.fill_(123.0)
    b.replay()
    assert torch.equal(b.u, eager)
    b.replay()
    assert torch.equal(b.u, eager)


def test_batch_benchmark_sizes_sample(cuda):
    """A sample of the 512-instance benchmark batch (sides 64..512, c in
    [0.5, 2]): every instance reaches rel err <= 1e-5 against the FP64
    oracle after 2 epochs (instances with c near 2 run at CFL near 1, where
    the FP32 forward substitution loses the most digits)."""
    from odil_gb300.batch import WaveBatch
    from odil_gb300.workloads import wave_batch_instances
    insts = wave_batch_instances(count=512)[:40]
    b = WaveBatch(insts, device=cuda)
    b.solve_mixed()
    errs = [W.rel_err(u, _oracle(inst)) for inst, u in zip(insts, b.unpack())]
    assert max(errs) <= 1e-5, max(errs)


def test_batch_rhs_kernels_match_single_instance(cuda):
    """The batched right-hand-side kernels (initial, float-pair) give, per
    instance, what the single-instance kernels give."""
    from odil_gb300.batch import WaveBatch
    from odil_gb300.wave import WaveKernels
    insts = _small_batch()
    b = WaveBatch(insts, device=cuda)
    rng = np.random.default_rng(3)
    hi = torch.as_tensor(rng.standard_normal(b.total), dtype=torch.float32,
                         device=cuda)
    lo = torch.as_tensor(1e-7 * rng.standard_normal(b.total),
                         dtype=torch.float32, device=cuda)
    r0 = torch.zeros(b.total, dtype=torch.float32, device=cuda)
    r1 = torch.zeros_like(r0)
    b.initial_rhs(r0)
    b.pair_residual(hi, lo, r1)
    for inst, off, (nt, nx) in zip(insts, b.offsets, b.shapes):
        k = WaveKernels(nt, nx, inst["dt"], inst["dx"], inst["c"],
                        inst["init_u"], inst["init_ut"], inst["left_u"],
                        inst["right_u"], device=cuda)
        sl = slice(off, off + nt * nx)
        e0 = torch.empty((nt, nx), dtype=torch.float32, device=cuda)
        k.initial_rhs(e0)
        assert torch.equal(r0[sl].view(nt, nx), e0)
        e1 = torch.empty_like(e0)
        k.pair_residual(hi[sl].view(nt, nx).contiguous(),
                        lo[sl].view(nt, nx).contiguous(), e1)
        assert torch.equal(r1[sl].view(nt, nx), e1)


def test_batch_three_epochs(cuda):
    """Three epochs (the third correction accumulates into lo)."""
    from odil_gb300.batch import WaveBatch
    insts = _small_batch()
    b = WaveBatch(insts, device=cuda)
    b.solve_mixed(epochs=3)
    for inst, u in zip(insts, b.unpack()):
        assert W.rel_err(u, _oracle(inst)) <= 1e-10, (inst["nt"], inst["c"])


@pytest.mark.parametrize("sides", [(5, 70), (120, 300), (1, 4)])
def test_batch_loss_grad_matches_single_instance_and_oracle(cuda, sides):
    """The one-launch fused loss + adjoint of the batch gives, per
    instance, the single-instance fused kernel's loss and gradient (FP32)
    and the oracle's FP64 values (util_op.py:627-654) to FP32 accuracy.
    Sides 5-70: one column strip per instance; 120-300: two or three
    strips (strip edges inside the grid); 1-4: grids of one to four
    columns (nx = 1 takes the general per-cell path)."""
    from odil_gb300.batch import WaveBatch
    from odil_gb300.wave import WaveKernels
    from odil_gb300.workloads import wave_batch_instances
    insts = _small_batch() if sides == (5, 70) else wave_batch_instances(
        count=8, seed=sides[1], nmin=sides[0], nmax=sides[1])
    b = WaveBatch(insts, device=cuda)
    rng = np.random.default_rng(5)
    u = torch.as_tensor(0.1 * rng.standard_normal(b.total),
                        dtype=torch.float32, device=cuda)
    g = torch.full_like(u, float("nan"))
    total, _ = b.loss_grad(u, g)
    losses = b.loss_inst.cpu().numpy()
    assert abs(total.item() - losses.sum()) <= 1e-12 * losses.sum()
    for q, (inst, off, (nt, nx)) in enumerate(zip(insts, b.offsets,
                                                  b.shapes)):
        sl = slice(off, off + nt * nx)
        uq = u[sl].view(nt, nx).contiguous()
        k = WaveKernels(nt, nx, inst["dt"], inst["dx"], inst["c"],
                        inst["init_u"], inst["init_ut"], inst["left_u"],
                        inst["right_u"], device=cuda)
        l1, g1 = k.loss_grad(uq)
        gq = g[sl].view(nt, nx)
        assert abs(losses[q] - l1.item()) <= 1e-5 * l1.item()
        assert float((gq - g1).abs().max()) <= 1e-4 * float(g1.abs().max())
        s = W.WaveSetup(nt, nx, inst["init_u"], inst["init_ut"],
                        inst["left_u"], inst["right_u"], c=inst["c"])
        lo, go = W.loss_grad(s, uq.double().cpu().numpy())
        assert abs(losses[q] - lo) <= 1e-4 * lo
        assert np.abs(gq.double().cpu().numpy() - go).max() <= \
            1e-3 * np.abs(go).max()


def test_batch_lbfgs_stage_then_newton_refinement(cuda):
    """The batch's FP32 fused-adjoint L-BFGS stage keeps the summed loss
    (it cannot lower it at FP32 resolution on this problem), and FP64
    Newton refinement from its iterate brings every instance to rel err
    <= 1e-5 against the FP64 oracle."""
    from odil_gb300.batch import WaveBatch
    from odil_gb300.workloads import wave_batch_instances
    insts = wave_batch_instances(count=512)[:24]
    b = WaveBatch(insts, device=cuda)
    g = torch.empty(b.total, dtype=torch.float32, device=cuda)
    l0 = b.loss_grad(torch.zeros_like(g), g)[0].item()
    x, info = b.lbfgs_warm_start(iters=10, m=5)
    assert info.epochs == 10
    # FP32 L-BFGS barely moves this loss (kappa(J^T J) ~ 1e10): it may not
    # rise beyond the approximate-Wolfe tolerance of 1e-6 of itself.
    assert b.loss_grad(x, g)[0].item() <= l0 * (1 + 1e-6)
    b.refine(x.double(), epochs=3)
    errs = [W.rel_err(u, _oracle(inst)) for inst, u in zip(insts, b.unpack())]
    assert max(errs) <= 1e-5, max(errs)


@pytest.mark.parametrize("sides", [(5, 70), (120, 300), (1, 4)])
def test_batch_persistent_solve_equals_multi_launch(cuda, sides):
    """The whole-batch mixed Newton in one persistent launch (right-hand
    sides formed inside the marches) gives bitwise the multi-launch
    sequence's solution for 1, 2 and 3 epochs, with every launch shape
    (columns per thread 1 with ring depth 8 and 16; 2 and 4 with 8), twice
    in a row (the work queue resets itself), and meets the oracle."""
    from odil_gb300.batch import WaveBatch
    from odil_gb300.workloads import wave_batch_instances
    insts = _small_batch() if sides == (5, 70) else wave_batch_instances(
        count=10, seed=sides[1], nmin=sides[0], nmax=sides[1])
    b = WaveBatch(insts, device=cuda)
    shapes = []
    for cpt in (1, 2, 4):
        threads = max(32, ((b.max_nx + cpt - 1) // cpt + 31) // 32 * 32)
        for pf in ((8, 16) if cpt == 1 else (8,)):
            shapes.append({"threads": threads, "cpt": cpt, "pf": pf,
                           "blocks_per_sm": 2})
    for ep in (1, 2, 3):
        ref = b.solve_mixed(epochs=ep).clone()
        for cfg in shapes:
            for _ in range(2):
                b.u.fill_(float("nan"))
                got = b.solve_persistent(epochs=ep, cfg=cfg)
                assert torch.equal(got, ref), (ep, cfg)
    if sides[0] > 1:
        for inst, u in zip(insts, b.unpack()):
            assert W.rel_err(u, _oracle(inst)) <= 1e-8, (inst["nt"], inst["c"])


def test_full_batch_every_instance_meets_the_oracle(cuda):
    """The configured 512-instance batch (sides 64-512, c in [0.5, 2]):
    mixed Newton (2 epochs) in one graph of launches and in one persistent
    launch; every instance, not just the largest error that a NaN-blind
    maximum would report, is within 1e-5 of the FP64 oracle, and the two
    launch forms agree bitwise on the instance cells."""
    from odil_gb300.batch import WaveBatch
    from odil_gb300.workloads import wave_batch_instances
    insts = wave_batch_instances(count=512)
    b = WaveBatch(insts, device=cuda)
    u_multi = b.solve_mixed(epochs=2).clone()
    got = b.unpack(u_multi)
    bad = []
    for q, (inst, u) in enumerate(zip(insts, got)):
        err = W.rel_err(u, _oracle(inst))
        if not err <= 1e-5:
            bad.append((q, inst["nt"], inst["nx"], inst["c"], err))
    assert not bad, bad[:5]
    b.solve_persistent(epochs=2)
    for u1, u2 in zip(got, b.unpack()):
        assert np.array_equal(u1, u2)
