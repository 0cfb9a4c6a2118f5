"""Sweep checkpoint files on the CPU: the manifest that ties a directory to
one sweep, the per-frequency records and their reload into the result
arrays (the GPU side, stopping and resuming a sweep, is in
test_gpu_sweep.py)."""
import os

import numpy as np
import pytest


def test_checkpoint_round_trip(bem, tmp_path):
    d = str(tmp_path / "ck")
    man = {"n": 4, "R": 2, "freqs": [100.0, 200.0, 300.0], "key": "abc"}
    names = bem.checkpoint_open(d, man)
    assert names == ["freq_00000.npz", "freq_00001.npz", "freq_00002.npz"]
    rng = np.random.default_rng(3)
    ps = rng.standard_normal((4, 2)) + 1j * rng.standard_normal((4, 2))
    info = bem.SolveInfo(iterations=17, rel_residual=3e-11, status=4, t_total=0.25)
    bem.checkpoint_write(d, names[1], ps, 200.0, info)
    # a half-written file under its temporary name is not a result
    open(os.path.join(d, names[2] + ".tmp123"), "wb").write(b"partial")
    p = np.zeros((4, 2, 3), np.complex128, order="F")
    infos = (bem.SolveInfo * 3)()
    solved = bem.checkpoint_load(d, bem.checkpoint_open(d, man), p, infos)
    assert solved.tolist() == [0, 1, 0]
    assert np.array_equal(p[:, :, 1], ps) and not p[:, :, 0].any() and not p[:, :, 2].any()
    assert infos[1].iterations == 17 and infos[1].status == 4
    assert infos[1].rel_residual == 3e-11 and infos[1].t_total == 0.25
    assert infos[0].iterations == 0


@pytest.mark.parametrize("field,value", [("key", "other"), ("R", 3), ("freqs", [100.0, 200.0])])
def test_checkpoint_of_another_sweep_is_refused(bem, tmp_path, field, value):
    d = str(tmp_path / "ck")
    man = {"n": 4, "R": 2, "freqs": [100.0, 200.0, 300.0], "key": "abc"}
    bem.checkpoint_open(d, man)
    with pytest.raises(ValueError):
        bem.checkpoint_open(d, {**man, field: value})
