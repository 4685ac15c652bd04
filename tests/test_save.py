"""Host checks of the ensemble writer's dispatch (no GPU): a state on a
SimpleGeometry is written as the device writer's text (SimpleState::saveToFile,
SimpleState.hpp:160-188), byte for byte; other geometries keep the exact
values as a binary .npy."""
import numpy as np
import torch

from metada_gb300 import algorithms as alg


def test_simple_state_goes_through_the_device_writer(tmp_path, monkeypatch):
    seen = []

    def fake_writer(values, nx, ny):
        seen.append((values, nx, ny))
        return b"   -0.000000     1.000000\n"

    monkeypatch.setattr(alg.K, "format_state", fake_writer)
    v = torch.tensor([-0.0, 1.0], dtype=torch.float64)
    path = tmp_path / "out" / "an_mean.txt"
    alg._save_state(path, v, alg.SimpleGeometry(2, 1))
    assert path.read_bytes() == b"   -0.000000     1.000000\n"
    assert len(seen) == 1 and seen[0][0] is v and seen[0][1:] == (2, 1)


def test_other_geometries_keep_exact_binary_values(tmp_path):
    v = torch.tensor([0.1, -0.0, 1e300, 2.0 ** -1074, 1.0 / 3.0], dtype=torch.float64)
    alg._save_state(tmp_path / "an_mean.nc", v, alg.LatLonGeometry(5, 1))
    back = np.load(tmp_path / "an_mean.npy")
    assert np.array_equal(back, v.numpy()) and np.signbit(back[1])
