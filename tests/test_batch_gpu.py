"""Batched Pennes ensemble (C ABI, CUDA): every instance against the CPU
oracle of the MRI-form Pennes update (examples/MRIDataPBHEqnFDM/
MRIDataPBHEqnFDM.hpp:143-169, pinned to the reference by the golden
vectors), the persistent work-queue path against the per-instance looped
path, and the autotuner.  Tolerance: relative max-norm 1e-12 (f64, f32x2)."""
from __future__ import annotations

import numpy as np
import pytest

import cases
import oracle as O
from masterthesis_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def small_ensemble(n_inst=7, seed=3):
    return W.pennes_ensemble(n_inst=n_inst, seed=seed, sizes=(3, 4, 7, 9, 17, 33, 40))


def oracle_run(spec, T):
    n = spec["n"]
    g = O.make_grid(n, tau=spec["tau"])
    shape = (n[2], n[1], n[0])
    u0 = np.full(shape, W.T_ARTERIAL)
    gb = np.full(shape, W.T_ARTERIAL)
    return O.pennes_mri(g, u0, T, 1.0, 1.0, spec["k"], 1.0, 1.0, spec["w_b"], W.T_ARTERIAL, spec["q"], gb)


def make_batch(M, specs, prec):
    b = M.Batch([W.pennes_batch_instance(s) for s in specs], precision=prec)
    for i, s in enumerate(specs):
        shape = (s["n"][2], s["n"][1], s["n"][0])
        b.upload(i, M.FIELD_F_A, W.pennes_source(s))
        b.upload(i, M.FIELD_U, np.full(shape, W.T_ARTERIAL))
    return b


@pytest.mark.parametrize("prec", ["f64", "f32x2"])
def test_batch_matches_oracle_per_instance(gpu, prec):
    M = gpu
    specs = small_ensemble()
    T = 25
    with make_batch(M, specs, prec) as b:
        b.step(T)
        for i, s in enumerate(specs):
            assert cases.rel_err(b.download(i), oracle_run(s, T)) <= 1e-12, (i, s["n"])


@pytest.mark.parametrize("prec", ["f64", "f32x2"])
def test_batch_queue_equals_batch(gpu, prec):
    """scafes_gpu_batch_create / _enqueue / _run: the instances enqueued one
    by one give the scafes_batch results bit for bit, across two runs; a
    late enqueue is refused."""
    M = gpu
    specs = small_ensemble(n_inst=5, seed=6)
    with make_batch(M, specs, prec) as b:
        b.step(9)
        b.step(4)
        want = [b.download(i) for i in range(len(specs))]
    with M.BatchQueue(prec) as q:
        for i, s in enumerate(specs):
            shape = (s["n"][2], s["n"][1], s["n"][0])
            assert q.enqueue(W.pennes_batch_instance(s), np.full(shape, W.T_ARTERIAL), W.pennes_source(s)) == i
        q.run(9)
        q.run(4)
        for i in range(len(specs)):
            assert np.array_equal(q.download(i), want[i]), i
        s = specs[0]
        with pytest.raises(M.ScafesError):
            q.enqueue(W.pennes_batch_instance(s), np.zeros((s["n"][2], s["n"][1], s["n"][0])))
    with M.BatchQueue(prec) as q:
        with pytest.raises(M.ScafesError):
            q.run(1)                                    # nothing enqueued


@pytest.mark.parametrize("prec", ["f32x2", "f32"])
def test_batch_deviation_form_round_trips(gpu, prec):
    """The FP32-based types hold u - g and F + fshift on the device (g the
    Dirichlet value): uploads and downloads give back the caller's values, a
    source that is never uploaded reads as 0 (to the element type's
    precision of the offset), and the results match FP64
    (1e-12 for pairs, 2e-5 for FP32 -- their usual bounds)."""
    M = gpu
    specs = small_ensemble(n_inst=4, seed=9)
    tol = 1e-12 if prec == "f32x2" else 2e-5
    with M.Batch([W.pennes_batch_instance(s) for s in specs], precision=prec) as b, \
            M.Batch([W.pennes_batch_instance(s) for s in specs], precision="f64") as r:
        for i, s in enumerate(specs):
            shape = (s["n"][2], s["n"][1], s["n"][0])
            u0 = np.full(shape, W.T_ARTERIAL) + np.random.default_rng(i).uniform(-0.5, 0.5, shape)
            b.upload(i, M.FIELD_U, u0)
            r.upload(i, M.FIELD_U, u0)
            if prec == "f32x2":
                assert cases.rel_err(b.download(i), u0) <= 1e-15
            # the source offset round-trips to pair (FP32) precision of fshift
            assert np.max(np.abs(b.download(i, M.FIELD_F_A))) <= (1e-14 if prec == "f32x2" else 1e-6)
        b.step(40)
        r.step(40)
        for i in range(len(specs)):
            assert cases.rel_err(b.download(i), r.download(i)) <= tol, i


def test_batch_equals_looped_and_all_schedules(gpu):
    M = gpu
    specs = small_ensemble(n_inst=9, seed=4)
    T = 13
    with make_batch(M, specs, "f64") as ref:
        ref.step_looped(T)
        want = [ref.download(i) for i in range(len(specs))]
    for tile in (1, 2, 3, 4):
        for ctas in (0, 1, 3):
            with make_batch(M, specs, "f64") as b:
                b.set_schedule(tile, ctas)
                b.step(T)
                for i in range(len(specs)):
                    assert np.array_equal(b.download(i), want[i]), (tile, ctas, i)


@pytest.mark.parametrize("prec", ["f64", "f32x2"])
def test_batch_depth2_equals_looped(gpu, prec):
    """Temporal depth 2 (two steps per pass over each instance, the plain
    sweep's depth-2 kernel on parallel graph chains; an odd last step at
    depth 1) gives the looped single-step results bit for bit."""
    M = gpu
    specs = small_ensemble(n_inst=9, seed=4)
    T = 13
    with make_batch(M, specs, prec) as ref:
        ref.step_looped(T)
        want = [ref.download(i) for i in range(len(specs))]
    with make_batch(M, specs, prec) as b:
        b.set_temporal_depth(2)
        b.step(T)
        assert b.info()["launches"] == 6 * len(specs) + 1
        for i in range(len(specs)):
            assert np.array_equal(b.download(i), want[i]), i
        with pytest.raises(M.ScafesError):
            b.set_temporal_depth(3)


@pytest.mark.parametrize("prec", ["f64", "f32x2"])
def test_batch_depth2_odd_pass_counts(gpu, prec):
    """Depth 2 over calls with an odd number of passes (step(10) = 5 passes,
    then step(2) = 1, then step(3) = 1 pass and a single step), each graph
    captured and replayed with both iterate parities: bit for bit the
    looped single-step results, on the small instances (3 and 4 nodes on
    an axis) of the graph-replay test."""
    M = gpu
    specs = small_ensemble(n_inst=5, seed=5)
    seq = [10, 2, 3, 10, 10]
    with make_batch(M, specs, prec) as ref:
        ref.step_looped(sum(seq))
        want = [ref.download(i) for i in range(len(specs))]
    with make_batch(M, specs, prec) as b:
        b.set_temporal_depth(2)
        for t in seq:
            b.step(t)
        for i in range(len(specs)):
            assert np.array_equal(b.download(i), want[i]), i


def test_batch_graph_replay_and_autotune(gpu):
    M = gpu
    specs = small_ensemble(n_inst=5, seed=5)
    with make_batch(M, specs, "f64") as b:
        tile, ctas = b.autotune(3)
        assert 1 <= tile <= 4 and ctas in (0, 1, 2, 4)
        d = b.temporal_depth()
        assert d["ms_depth1"] > 0.0 and d["ms_depth2"] > 0.0  # both depths measured
        assert d["depth"] == (2 if d["ms_depth2"] < d["ms_depth1"] else 1)
        b.step(10)   # captures the graph for 10 steps
        b.step(10)   # replays it (other buffer parity: second graph)
        b.step(10)   # replays the first graph
        got = [b.download(i) for i in range(len(specs))]
    for i, s in enumerate(specs):
        assert cases.rel_err(got[i], oracle_run(s, 30)) <= 1e-12


def test_batch_errors(gpu):
    M = gpu
    specs = small_ensemble(n_inst=2)
    with make_batch(M, specs, "f64") as b:
        with pytest.raises(M.ScafesError):
            b.upload(5, M.FIELD_U, np.zeros(8))
        with pytest.raises(M.ScafesError):
            b.upload(0, M.FIELD_U, np.zeros(3))
        with pytest.raises(M.ScafesError):
            b.set_schedule(9, 0)
