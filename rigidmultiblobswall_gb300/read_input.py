"""Input files of the reference's drivers (read_input/read_input.py:8-160):
'key value' lines, '#' comments, repeated 'structure' / 'obstacle' /
'articulated' lines numbered in order, the same attribute names and
defaults, structure IDs from the clones file names, and the restart rule:
with initial_step > 0 each structure's clones file becomes
<output_name>.<ID>.<initial_step:08d>.clones.

One key of this package's own: gb300_precision (fp64 | df64 | mixed, default
fp64), the arithmetic of the blob mobility products.
"""
import ntpath

import numpy as np


def _floats(text, default):
    return np.array([float(t) for t in (text or default).split()]) if (text or default) != "None" else np.array([])


class ReadInput:
    """Parsed input file (attribute names as the reference's ReadInput)."""

    _FLOATS = {"dt": 0.0, "eta": 1.0, "g": 1.0, "blob_radius": 1.0, "tracer_radius": 0.0, "kT": 1.0,
               "repulsion_strength_wall": 1.0, "debye_length_wall": 1.0, "repulsion_strength": 1.0,
               "debye_length": 1.0, "solver_tolerance": 1e-8, "nonlinear_solver_tolerance": 1e-8, "rf_delta": 1e-3,
               "repulsion_strength_firm": 0.0, "firm_delta": 1e-2, "Lub_Cut": 4.5, "zmin": 0.0, "zmax": 1e7,
               "diffusion_coefficient": 1.0}
    _INTS = {"n_steps": 0, "initial_step": 0, "n_save": 1, "n_relaxation": 0, "sample_HydroGrid": 1,
             "save_HydroGrid": 0, "hydro_interactions": 1, "update_PC": 1}
    _STRINGS = {"scheme": "deterministic_forward_euler", "output_name": "run",
                "mobility_blobs_implementation": "python", "mobility_vector_prod_implementation": "python",
                "blob_blob_force_implementation": "None", "body_body_force_torque_implementation": "None",
                "save_body_mobility": "False", "save_blobs_mobility": "False", "save_velocities": "False",
                "save_clones": "one_file_per_step", "free_kinematics": "True", "domain": "single_wall",
                "domType": "RPB", "gb300_precision": "fp64"}

    def __init__(self, entries):
        self.entries = entries
        self.input_file = entries
        self.options = {}
        counts = {"structure": 0, "obstacle": 0, "articulated": 0}
        with open(self.input_file, "r") as f:
            for line in f:
                if "#" in line:
                    line = line.split("#", 1)[0]
                line = line.strip()
                if not line:
                    continue
                option, value = line.split(None, 1)
                if option in counts:
                    kind = option
                    option = kind + str(counts[kind])
                    counts[kind] += 1
                self.options[option] = value
        o = self.options
        for k, d in self._FLOATS.items():
            setattr(self, k, float(o.get(k) or d))
        for k, d in self._INTS.items():
            setattr(self, k, int(o.get(k) or d))
        for k, d in self._STRINGS.items():
            setattr(self, k, str(o.get(k) or d))
        self.theta = float(o.get("tilt_angle") or 0.0)
        self.random_state = o.get("random_state")
        self.seed = o.get("seed")
        self.slip_file = o.get("slip_file")
        self.force_file = o.get("force_file")
        self.velocity_file = o.get("velocity_file")
        self.periodic_length = _floats(o.get("periodic_length"), "0 0 0")
        self.omega_one_roller = _floats(o.get("omega_one_roller"), "0 0 0")
        self.call_HydroGrid = str(o.get("call_HydroGrid") or "False") == "True"
        self.num_free_bodies = counts["structure"]
        self.structures, self.structures_ID = [], []
        self.articulated, self.articulated_ID = [], []
        for kind in ("structure", "obstacle"):
            for i in range(counts[kind]):
                self.structures.append(str(o.get(kind + str(i))).split())
        for i in range(counts["articulated"]):
            files = str(o.get("articulated" + str(i))).split()
            self.articulated_ID.append(ntpath.split(files[1])[1][:-7])
            self.articulated.append(files)
        for files in self.structures:
            self.structures_ID.append(ntpath.split(files[1])[1][:-7])
        if self.initial_step > 0:
            for k, files in enumerate(self.structures):
                files[1] = self.output_name + "." + self.structures_ID[k] + "." + str(self.initial_step).zfill(8) + \
                    ".clones"
