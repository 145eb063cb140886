"""Snapshot files (the reference's field output, src/ScaFES_Problem.hpp:
4254-4340, as raw FP64 records; read back as an initial iterate).

CPU: the reader against a file written here in the documented layout, and
its errors.  GPU: scafes_gpu_step_snapshots writes the iterate at the start,
every `interval` steps and at the end while the steps run; each snapshot
must equal the iterate a plain run downloads at that step (same kernels:
bit-exact), with the step and time of that step.
"""
from __future__ import annotations

import numpy as np
import pytest


def write_file(path, n, records):
    with open(path, "wb") as f:
        f.write(b"SCAFESS1")
        f.write(np.array([1, *n, 0, 0], dtype="<i4").tobytes())
        for step, time, a in records:
            f.write(np.array([step], dtype="<i8").tobytes())
            f.write(np.array([time], dtype="<f8").tobytes())
            f.write(np.ascontiguousarray(a, dtype="<f8").tobytes())


def test_snapshot_reader(native, tmp_path):
    M = native
    n = (5, 4, 3)
    rng = np.random.default_rng(1)
    recs = [(k * 7, 0.5 * k, rng.standard_normal((3, 4, 5))) for k in range(3)]
    p = tmp_path / "s.bin"
    write_file(p, n, recs)
    assert M.snapshot_info(p) == (n, 3)
    for k, (st, tm, a) in enumerate(recs):
        b, st2, tm2 = M.snapshot_read(p, k)
        assert np.array_equal(a, b) and st2 == st and tm2 == tm
    with pytest.raises(M.ScafesError):
        M.snapshot_read(p, 3)
    bad = tmp_path / "bad.bin"
    bad.write_bytes(b"not a snapshot file at all, definitely not")
    with pytest.raises(M.ScafesError):
        M.snapshot_info(bad)
    with pytest.raises(M.ScafesError):
        M.snapshot_info(tmp_path / "missing.bin")


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["f64", "f32x2", "f32"])
def test_snapshots_match_plain_run(gpu, tmp_path, prec):
    M = gpu
    n, T, every = (40, 30, 21), 10, 3
    tau = 0.9 / (2.0 * sum((m - 1) ** 2 for m in n))
    rng = np.random.default_rng(5)
    u0 = rng.uniform(-1.0, 1.0, (n[2], n[1], n[0]))
    cfg = M.make_cfg(n, tau=tau, t_start=0.25, precision=prec, heat=(1.0, 1.0, 0.0))
    path = tmp_path / "snap.bin"
    with M.Plain(cfg) as p:
        p.upload(M.FIELD_U, u0)
        p.step(2)                       # snapshots count absolute steps
        p.step_snapshots(T, every, path)
        final = p.download()
    steps = [2, 3, 6, 9, 12]            # start, multiples of 3, end
    assert M.snapshot_info(path) == (n, len(steps))
    with M.Plain(cfg) as q:
        q.upload(M.FIELD_U, u0)
        done = 0
        for k, s in enumerate(steps):
            q.step(s - done)
            done = s
            a, st, tm = M.snapshot_read(path, k)
            assert st == s and tm == pytest.approx(0.25 + s * tau, rel=1e-15)
            assert np.array_equal(a, q.download()), (prec, s)
    assert np.array_equal(final, a)
