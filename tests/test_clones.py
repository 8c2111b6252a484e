"""CPU: structure-file reading and trajectory I/O (clones.py) against the
reference's read_clones_file / read_vertex_file outputs and the text its
driver writes (tests/golden/clones.npz), bit-exact; and the save cadence of the
time-stepping loop and its resume, on a stand-in integrator."""
import os

import numpy as np
import pytest

from conftest import golden
from rigidmultiblobswall_gb300 import clones


def _write(tmp_path, name, text):
    p = os.path.join(str(tmp_path), name)
    with open(p, "w") as f:
        f.write(str(text))
    return p


@pytest.mark.parametrize("key", ["shell12", "boomerang15", "synthetic"])
def test_read_clones_file_matches_reference(tmp_path, key):
    g = golden("clones.npz")
    n, loc, ori = clones.read_clones_file(_write(tmp_path, "a.clones", g[key + "_clones_text"]))
    assert n == g[key + "_n"][0]
    np.testing.assert_array_equal(loc, g[key + "_locations"])
    np.testing.assert_array_equal(ori, g[key + "_orientations"])


@pytest.mark.parametrize("key", ["shell12", "boomerang15"])
def test_read_vertex_file_matches_reference(tmp_path, key):
    g = golden("clones.npz")
    r = clones.read_vertex_file(_write(tmp_path, "a.vertex", g[key + "_vertex_text"]))
    np.testing.assert_array_equal(r, g[key + "_vertex"])


def test_written_text_matches_reference_driver():
    g = golden("clones.npz")
    assert clones.format_clones(g["write_locations"], g["write_orientations"]) == str(g["write_text"])


def test_config_round_trip_is_bit_exact(tmp_path):
    g = golden("clones.npz")
    p = os.path.join(str(tmp_path), "run.body.config")
    rng = np.random.default_rng(1)
    frames = [(rng.standard_normal((4, 3)) * 10.0 ** rng.integers(-12, 12, (4, 3)), rng.standard_normal((4, 4)))
              for _ in range(3)]
    frames.append((g["write_locations"][:4], g["write_orientations"][:4]))
    with open(p, "w") as f:
        for loc, ori in frames:
            f.write(clones.format_clones(loc, ori))
    back = clones.read_config_file(p)
    assert len(back) == len(frames)
    for (l0, o0), (l1, o1) in zip(frames, back):
        np.testing.assert_array_equal(l0, l1)
        np.testing.assert_array_equal(o0, o1)
    l, o = clones.resume_state(p)
    np.testing.assert_array_equal(l, frames[-1][0])


class _Stepper:
    """Stand-in integrator: deterministic host-side state updates."""

    def __init__(self, x, q):
        import torch
        self.x = torch.as_tensor(x, dtype=torch.float64).clone()
        self.q = torch.as_tensor(q, dtype=torch.float64).clone()
        self.scheme = "stand_in"
        self.invalid_configuration_count = 0
        self.det_iterations_count = 0
        self.stoch_iterations_count = 0
        self.steps = []

    def advance_time_step(self, dt, step=None):
        self.steps.append(step)
        self.x = self.x + dt * (1.0 + 0.1 * self.x)
        self.q = self.q * 0.5 + 0.25 * self.q.roll(1, 1)
        self.det_iterations_count += 3


@pytest.mark.parametrize("save_clones", ["one_file_per_step", "one_file"])
def test_run_save_cadence_and_resume(tmp_path, save_clones):
    """Saves at step % n_save == 0 and after the last step (multi_bodies.py:1422-1457);
    a run resumed from a saved frame at initial_step continues identically."""
    rng = np.random.default_rng(2)
    x0, q0 = rng.standard_normal((5, 3)), rng.standard_normal((5, 4))
    out = os.path.join(str(tmp_path), "full")
    s = _Stepper(x0, q0)
    clones.run(s, 0.1, 7, n_save=3, output_name=out, structures_ID=["a", "b"], body_types=[2, 3],
               save_clones=save_clones)
    assert s.steps == list(range(7))
    saved = [0, 3, 6]  # 7 % 3 != 0: no save after the last step
    for ID, sl in (("a", slice(0, 2)), ("b", slice(2, 5))):
        if save_clones == "one_file_per_step":
            names = sorted(f for f in os.listdir(str(tmp_path)) if f.startswith("full." + ID + "."))
            assert names == ["full.%s.%08d.clones" % (ID, k) for k in saved]
        else:
            assert len(clones.read_config_file(out + "." + ID + ".config")) == len(saved)
    info = open(out + ".info").read()
    assert "deterministic_iterations_count = 21" in info
    # straight 6 steps vs 3 steps + resume from the saved step-3 frame
    s6 = _Stepper(x0, q0)
    clones.run(s6, 0.1, 6, n_save=3, output_name=os.path.join(str(tmp_path), "six"), save_clones=save_clones)
    first = _Stepper(x0, q0)
    clones.run(first, 0.1, 3, n_save=3, output_name=os.path.join(str(tmp_path), "p1"), save_clones=save_clones)
    src = (os.path.join(str(tmp_path), "p1.body.00000003.clones") if save_clones == "one_file_per_step"
           else os.path.join(str(tmp_path), "p1.body.config"))
    loc, ori = clones.resume_state(src)
    np.testing.assert_array_equal(loc, first.x.numpy())
    second = _Stepper(loc, first.q.numpy())
    clones.run(second, 0.1, 6, n_save=3, output_name=os.path.join(str(tmp_path), "p2"), initial_step=3,
               save_clones=save_clones)
    assert second.steps == [3, 4, 5]
    np.testing.assert_array_equal(second.x.numpy(), s6.x.numpy())


@pytest.mark.parametrize("tag", ["input", "restart"])
def test_read_input_matches_reference(tmp_path, tag):
    """ReadInput against the reference's parse of the same file (values as the
    reference's str() of each attribute; restart rewrites the clones paths)."""
    from rigidmultiblobswall_gb300.read_input import ReadInput
    g = golden("clones.npz")
    rd = ReadInput(_write(tmp_path, tag + ".dat", g[tag + "_text"]))
    for k, v in zip(g["input_keys"], g[tag + "_values"]):
        assert str(getattr(rd, str(k))) == str(v), k
    np.testing.assert_array_equal(rd.periodic_length, g[tag + "_periodic_length"])
    assert [" ".join(s) for s in rd.structures] == [str(s) for s in g[tag + "_structures"]]
    assert rd.structures_ID == [str(s) for s in g[tag + "_structures_ID"]]
    assert rd.gb300_precision == "fp64"
