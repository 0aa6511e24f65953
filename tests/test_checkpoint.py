"""Checkpoint files and the reference's text dump (CPU)."""
from __future__ import annotations

import numpy as np
import pytest

from ads_gb300 import checkpoint


def test_binary_round_trip(tmp_path):
    u = np.random.default_rng(0).standard_normal(5 * 4 * 3)
    p = tmp_path / "s.ckp"
    checkpoint.save(p, u, (5, 4, 3), degrees=(2, 2, 3), step=17, dt=1e-6, t=1.7e-5)
    v, info = checkpoint.load(p)
    np.testing.assert_array_equal(u, v)
    assert info == {"ndim": 3, "shape": (5, 4, 3), "degrees": (2, 2, 3), "step": 17, "dt": 1e-6, "t": 1.7e-5}
    raw = open(p, "rb").read()
    assert raw[:8] == b"ADSGCKP1" and len(raw) == 56 + 8 * u.size
    assert np.frombuffer(raw[56:], "<f8")[7] == u[7]  # x-fastest, little-endian doubles


def test_bad_files_are_rejected(tmp_path):
    p = tmp_path / "bad"
    p.write_bytes(b"NOTACKPT" + bytes(60))
    with pytest.raises(ValueError):
        checkpoint.load(p)
    checkpoint.save(tmp_path / "t", np.zeros(6), (2, 3))
    data = (tmp_path / "t").read_bytes()
    (tmp_path / "t2").write_bytes(data[:-8])
    with pytest.raises(ValueError):
        checkpoint.load(tmp_path / "t2")
    with pytest.raises(ValueError):
        checkpoint.save(tmp_path / "t3", np.zeros(5), (2, 3))


def test_text_dump_round_trip(tmp_path):
    u = np.random.default_rng(1).standard_normal(4 * 3)
    p = tmp_path / "u.data"
    checkpoint.write_text(p, u, (4, 3))
    first = open(p).readline().split()
    assert first[:2] == ["0", "0"] and float(first[2]) == u[0]
    np.testing.assert_array_equal(checkpoint.read_text(p, (4, 3)), u)
    u3 = np.random.default_rng(2).standard_normal(2 * 3 * 4)
    checkpoint.write_text(tmp_path / "v", u3, (2, 3, 4))
    np.testing.assert_array_equal(checkpoint.read_text(tmp_path / "v", (2, 3, 4)), u3)
