"""GPU: the simulation driver (multi_bodies.main with an input file in the
reference's format) against the device integrator run by hand, and a run
resumed at initial_step from its saved clones files."""
import os

import numpy as np
import pytest

from conftest import golden
from rigidmultiblobswall_gb300 import clones, forces, integrator
from rigidmultiblobswall_gb300 import multi_bodies as mbs
from rigidmultiblobswall_gb300.rigid import RigidSystem

pytestmark = pytest.mark.gpu


def write_case(d, scheme, n_steps, extra=""):
    g = golden("rigid.npz")
    ref = g["s12_ref_cfg"]
    a = float(g["s12_params"][0])
    locs, quats = g["s12_locs"][:4], g["s12_quats"][:4]
    vtx = os.path.join(d, "shell.vertex")
    with open(vtx, "w") as f:
        f.write("%d\n" % ref.shape[0] + "".join("%r %r %r\n" % tuple(float(c) for c in p) for p in ref))
    cl = os.path.join(d, "shell.clones")
    clones.write_clones_file(cl, locs, quats)
    inp = os.path.join(d, "run.dat")
    with open(inp, "w") as f:
        f.write("scheme %s\ndt 0.01\nn_steps %d\nn_save 2\neta 1.0\ng 1.0\nblob_radius %r\nkT 0.5\n"
                "repulsion_strength_wall 0.3\ndebye_length_wall %r\nblob_blob_force_implementation python\n"
                "repulsion_strength 0.3\ndebye_length %r\nsolver_tolerance 1e-10\nseed 11\n"
                "output_name %s\nstructure %s %s\n%s" % (scheme, n_steps, a, 0.1 * a, 0.1 * a,
                                                         os.path.join(d, "out", "run"), vtx, cl, extra))
    return inp, ref, a, locs, quats


def test_driver_matches_integrator(cuda_device, tmp_path):
    d = str(tmp_path)
    inp, ref, a, locs, quats = write_case(d, "stochastic_traction_EM", 4, "save_clones one_file\n")
    mbs.main(["--input-file", inp])
    frames = clones.read_config_file(os.path.join(d, "out", "run.shell.config"))
    assert len(frames) == 3
    sys_ = RigidSystem([ref.shape[0]] * 4, 1.0, a)
    it = integrator.QuaternionIntegrator(sys_, "stochastic_traction_EM", locs, quats, np.tile(ref, (4, 1)),
                                         tolerance=1e-10, kT=0.5, seed=11)
    kw = dict(g=1.0, repulsion_strength_wall=0.3, debye_length_wall=0.1 * a, repulsion_strength=0.3,
              debye_length=0.1 * a, periodic_length=np.zeros(3))
    it.force_torque_calculator = lambda s, r: forces.force_torque_calculator_sort_by_bodies(s, r, **kw)
    for step in range(4):
        it.advance_time_step(0.01)
    np.testing.assert_allclose(frames[-1][0], it.x.cpu().numpy(), rtol=0, atol=1e-12)
    np.testing.assert_allclose(frames[-1][1], it.q.cpu().numpy(), rtol=0, atol=1e-12)
    info = open(os.path.join(d, "out", "run.info")).read()
    assert "stochastic_iterations_count" in info
    assert os.path.exists(os.path.join(d, "out", "run.bodies_info"))


def test_driver_resumes_at_initial_step(cuda_device, tmp_path):
    d = str(tmp_path)
    inp, *_ = write_case(d, "deterministic_forward_euler", 4)
    mbs.main(["--input-file", inp])
    full = clones.read_clones_file(os.path.join(d, "out", "run.shell.00000004.clones"))
    inp2, *_ = write_case(d, "deterministic_forward_euler", 2)
    mbs.main(["--input-file", inp2])
    inp3, *_ = write_case(d, "deterministic_forward_euler", 4, "initial_step 2\n")
    mbs.main(["--input-file", inp3])
    resumed = clones.read_clones_file(os.path.join(d, "out", "run.shell.00000004.clones"))
    np.testing.assert_allclose(resumed[1], full[1], rtol=0, atol=1e-12)
    np.testing.assert_allclose(resumed[2], full[2], rtol=0, atol=1e-12)
