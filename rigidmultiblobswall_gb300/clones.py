"""Trajectory I/O and the time-stepping loop of the reference's multi_bodies
driver, around the device integrator (integrator.QuaternionIntegrator).

* read_vertex_file   read_input/read_vertex_file.py:8-34 (body-frame blob coordinates)
* read_clones_file   read_input/read_clones_file.py:12-50 (number of bodies, locations,
                     normalised quaternions)
* write_clones_file / format_clones
                     the per-body line '%s %s %s %s %s %s %s' of location and
                     quaternion, after a line with the body count
                     (multi_bodies/multi_bodies.py:1428-1457)
* read_config_file   the 'one_file' trajectory (<output>.<ID>.config): one such
                     block per saved step
* run                the loop of multi_bodies/multi_bodies.py:1414-1627: save at
                     every step % n_save == 0 (and after the last step), advance,
                     write <output>.time and <output>.info; initial_step > 0
                     resumes a run from a saved configuration
* resume_state       a saved frame (a .clones file or a frame of a .config
                     file) as the state to resume from

Locations and quaternions are host numpy arrays here; the integrator's state
is copied from the device only at the saved steps.  Numbers are written as
Python's shortest round-trip representation of the float64 (what '%s' prints
for the reference's numpy float64), so a saved frame reads back bit-exactly.
"""
import os
import time

import numpy as np


def _data_lines(name_file):
    """Non-empty lines with '#' comments removed."""
    with open(name_file, "r") as f:
        for line in f:
            if "#" in line:
                line = line.split("#", 1)[0]
            line = line.strip()
            if line:
                yield line


def read_vertex_file(name_file):
    """(Nblobs, 3) blob coordinates of a .vertex file: a count line, then one
    'x y z' line per blob (every following data line is read)."""
    coor = []
    for i, line in enumerate(_data_lines(name_file)):
        if i == 0:
            int(line.split()[0])
            continue
        coor.append(np.array([float(t) for t in line.split()]))
    return np.array(coor)


def read_clones_file(name_file):
    """(number_of_bodies, locations (Nb, 3), orientations (Nb, 4)) of a .clones
    file; quaternions are normalised, lines past the last body are ignored."""
    locations, orientations = [], []
    number_of_bodies = None
    for i, line in enumerate(_data_lines(name_file)):
        if i == 0:
            number_of_bodies = int(line.split()[0])
        else:
            data = line.split()
            locations.append([float(data[0]), float(data[1]), float(data[2])])
            q = np.array([float(data[3]), float(data[4]), float(data[5]), float(data[6])])
            orientations.append(q / np.linalg.norm(q))
        if number_of_bodies is not None and i == number_of_bodies:
            break
    return number_of_bodies, np.array(locations).reshape(-1, 3), np.array(orientations).reshape(-1, 4)


def format_clones(locations, orientations):
    """The body count line and one 'x y z s p1 p2 p3' line per body."""
    loc = np.asarray(locations, dtype=np.float64).reshape(-1, 3)
    ori = np.asarray(orientations, dtype=np.float64).reshape(-1, 4)
    lines = [str(loc.shape[0]) + "\n"]
    for x, q in zip(loc.tolist(), ori.tolist()):
        lines.append("%s %s %s %s %s %s %s\n" % (x[0], x[1], x[2], q[0], q[1], q[2], q[3]))
    return "".join(lines)


def write_clones_file(name_file, locations, orientations):
    with open(name_file, "w") as f:
        f.write(format_clones(locations, orientations))


def read_config_file(name_file):
    """Every frame of a 'one_file' trajectory: list of (locations, orientations);
    quaternions as written (not renormalised)."""
    frames = []
    lines = list(_data_lines(name_file))
    i = 0
    while i < len(lines):
        n = int(lines[i].split()[0])
        block = np.array([[float(t) for t in ln.split()[:7]] for ln in lines[i + 1:i + 1 + n]]).reshape(n, 7)
        if block.shape[0] != n:
            raise ValueError("truncated frame in %s" % name_file)
        frames.append((block[:, :3].copy(), block[:, 3:].copy()))
        i += 1 + n
    return frames


def resume_state(name_file, frame=-1):
    """(locations, orientations) to resume from: a .clones file, or frame
    `frame` of a .config trajectory."""
    if name_file.endswith(".config"):
        return read_config_file(name_file)[frame]
    _, loc, ori = read_clones_file(name_file)
    return loc, ori


class TrajectoryWriter:
    """Saves the bodies of each structure (consecutive groups of body_types[i]
    bodies, named structures_ID[i]) as <output_name>.<ID>.<step:08d>.clones
    ('one_file_per_step') or appended frames of <output_name>.<ID>.config
    ('one_file')."""

    def __init__(self, output_name, structures_ID, body_types, save_clones="one_file_per_step"):
        if save_clones not in ("one_file_per_step", "one_file"):
            raise ValueError("save_clones must be 'one_file_per_step' or 'one_file'")
        if len(structures_ID) != len(body_types):
            raise ValueError("one structure ID per body type")
        self.output_name = output_name
        self.structures_ID = list(structures_ID)
        self.body_types = [int(b) for b in body_types]
        self.save_clones = save_clones
        self.files = None
        if save_clones == "one_file":
            self.files = [open(output_name + "." + ID + ".config", "w") for ID in self.structures_ID]

    def save(self, step, locations, orientations):
        off = 0
        for i, ID in enumerate(self.structures_ID):
            nb = self.body_types[i]
            text = format_clones(locations[off:off + nb], orientations[off:off + nb])
            if self.save_clones == "one_file_per_step":
                with open(self.output_name + "." + ID + "." + str(step).zfill(8) + ".clones", "w") as f:
                    f.write(text)
            else:
                self.files[i].write(text)
                self.files[i].flush()
            off += nb

    def close(self):
        if self.files:
            for f in self.files:
                f.close()
            self.files = None


def run(integrator, dt, n_steps, n_save=1, output_name="run", structures_ID=("body",), body_types=None,
        save_clones="one_file_per_step", initial_step=0, verbose=False):
    """Advance `integrator` from step initial_step to n_steps, saving the
    configuration at every step % n_save == 0 and after the last step, as
    multi_bodies/multi_bodies.py:1414-1627 does; writes <output_name>.time
    (wall-clock seconds) and <output_name>.info (iteration and
    invalid-configuration counters)."""
    nb = integrator.x.shape[0]
    body_types = [nb] if body_types is None else list(body_types)
    if sum(body_types) != nb:
        raise ValueError("body_types must add up to the number of bodies")
    out_dir = os.path.dirname(output_name)
    if out_dir:
        os.makedirs(out_dir, exist_ok=True)
    writer = TrajectoryWriter(output_name, structures_ID, body_types, save_clones)
    start = time.time()

    def save(step):
        if verbose:
            print("Integrator = ", integrator.scheme, ", step = ", step, ", invalid configurations",
                  integrator.invalid_configuration_count, ", wallclock time = ", time.time() - start)
        writer.save(step, integrator.x.cpu().numpy(), integrator.q.cpu().numpy())

    step = initial_step - 1
    try:
        for step in range(initial_step, n_steps):
            if step % n_save == 0 and step >= 0:
                save(step)
            integrator.advance_time_step(dt, step=step)
        if (step + 1) % n_save == 0 and step >= 0:
            save(step + 1)
    finally:
        writer.close()
    with open(output_name + ".time", "w") as f:
        f.write(str(time.time() - start) + "\n")
    with open(output_name + ".info", "w") as f:
        f.write("invalid_configuration_count    = " + str(integrator.invalid_configuration_count) + "\n"
                + "deterministic_iterations_count = " + str(integrator.det_iterations_count) + "\n"
                + "stochastic_iterations_count    = " + str(integrator.stoch_iterations_count) + "\n"
                + "nonlinear_iterations_count     = 0\n")
