"""Drop-in for the rigid-body part of the reference's multi_bodies/multi_bodies.py.

Same names and argument meaning:

* get_blobs_r_vectors, calc_K_matrix_bodies           (multi_bodies.py:194-204, 306-316)
* K_matrix_vector_prod, K_matrix_T_vector_prod         (multi_bodies.py:328-371)
* linear_operator_rigid                                (multi_bodies.py:424-471)
* build_block_diagonal_preconditioner                  (multi_bodies.py:752-903)
* build_block_diagonal_preconditioners_det_stoch       (multi_bodies.py:480-618)

Every operator runs on the GPU (librmw_gb300) through a RigidSystem that is
cached per suspension shape and re-uploaded only when the configuration
changes.  numpy vectors in -> numpy vectors out (one copy each way per call,
like the reference's pycuda path); CUDA torch vectors stay on the device.

Not supported (raise NotImplementedError): constraints / articulated bodies and
prescribed kinematics - the rows the reference adds for them are absent in the
suspensions this package targets.
"""
import numpy as np

from .rigid import RigidSystem

_cache = {}


def _is_torch(x):
    return type(x).__module__.startswith("torch")


def _check_supported(bodies, constraints=None, articulated=None):
    if constraints:
        raise NotImplementedError("constraints are not supported")
    if articulated:
        raise NotImplementedError("articulated bodies are not supported")
    if any(getattr(b, "prescribed_kinematics", False) for b in bodies):
        raise NotImplementedError("prescribed kinematics are not supported")


def system_for(bodies, r_vectors, eta, a, periodic_length=None):
    """Cached RigidSystem for this list of bodies at this configuration."""
    counts = tuple(int(b.Nblobs) for b in bodies)
    L = np.zeros(3) if periodic_length is None else np.asarray(periodic_length, dtype=np.float64).reshape(3)
    key = (counts, float(eta), float(a), tuple(L.tolist()))
    entry = _cache.get(key)
    if entry is None:
        if len(_cache) > 8:
            _cache.clear()
        entry = {"sys": RigidSystem(counts, eta, a, periodic_length=L), "sig": None}
        _cache[key] = entry
    locs = np.array([b.location for b in bodies], dtype=np.float64)
    if _is_torch(r_vectors):
        sig = ("torch", r_vectors.data_ptr(), r_vectors._version, locs.tobytes())
    else:
        r_np = np.ascontiguousarray(r_vectors, dtype=np.float64)
        sig = ("np", r_np.tobytes(), locs.tobytes())
    if entry["sig"] != sig:
        entry["sys"].set_configuration(r_vectors, locs)
        entry["sig"] = sig
    return entry["sys"]


def _to_out(y, like):
    return y if _is_torch(like) else y.cpu().numpy()


def get_blobs_r_vectors(bodies, Nblobs):
    """Coordinates of all blobs, shape (Nblobs, 3)."""
    r_vectors = np.empty((Nblobs, 3))
    offset = 0
    for b in bodies:
        r_vectors[offset:offset + b.Nblobs] = b.get_r_vectors()
        offset += b.Nblobs
    return r_vectors


def calc_K_matrix_bodies(bodies, Nblobs):
    return [b.calc_K_matrix() for b in bodies]


def K_matrix_vector_prod(bodies, vector, Nblobs, K_bodies=None, eta=1.0, a=1.0):
    """K * vector, shape (Nblobs, 3)."""
    sys_ = system_for(bodies, get_blobs_r_vectors(bodies, Nblobs), eta, a)
    y = sys_.K_mult(vector)
    return _to_out(y, vector).reshape(Nblobs, 3)


def K_matrix_T_vector_prod(bodies, vector, Nblobs, K_bodies=None, eta=1.0, a=1.0):
    """K^T * vector, shape (2 Nbodies, 3)."""
    sys_ = system_for(bodies, get_blobs_r_vectors(bodies, Nblobs), eta, a)
    y = sys_.KT_mult(vector)
    return _to_out(y, vector).reshape(2 * len(bodies), 3)


def linear_operator_rigid(vector, bodies, constraints, r_vectors, eta, a, K_bodies=None, C_constraints=None,
                          *args, **kwargs):
    """|  M   -K ||lambda|   (multi_bodies.py:424-471), on the GPU.
       | -K^T  0 ||  U   |
    Extra keyword ``mode`` = 'fp64' (default) or 'mixed'."""
    _check_supported(bodies, constraints)
    sys_ = system_for(bodies, r_vectors, eta, a, kwargs.get("periodic_length"))
    y = sys_.apply(vector, mode=kwargs.get("mode", "fp64"))
    return _to_out(y, vector)


class _Applier:
    """Callable returned by the preconditioner builders (the reference returns
    functools.partial objects with the same call signature)."""

    def __init__(self, fn):
        self.fn = fn

    def __call__(self, vector, *args, **kwargs):
        return _to_out(self.fn(vector), vector)


def build_block_diagonal_preconditioner(bodies, articulated, r_vectors, Nblobs, eta, a, *args, **kwargs):
    """Block-diagonal preconditioner of the rigid mobility problem; returns a
    callable vector -> P^-1 vector (multi_bodies.py:752-903)."""
    _check_supported(bodies, None, articulated)
    sys_ = system_for(bodies, r_vectors, eta, a, kwargs.get("periodic_length"))
    sys_.build_pc(stochastic=False)
    return _Applier(sys_.apply_pc)


def build_block_diagonal_preconditioners_det_stoch(bodies, r_vectors, Nblobs, eta, a, *args, **kwargs):
    """(PC, mobility_pc, P_inv_mult) of multi_bodies.py:480-618: the block-diagonal
    preconditioner, w -> L^-1 M L^-T w and w -> L w with M_b = L L^T per body."""
    _check_supported(bodies)
    sys_ = system_for(bodies, r_vectors, eta, a, kwargs.get("periodic_length"))
    sys_.build_pc(stochastic=True)
    mode = kwargs.get("mode", "fp64")
    return (_Applier(sys_.apply_pc), _Applier(lambda w: sys_.mobility_pc(w, mode=mode)),
            _Applier(sys_.P_inv_mult))


# ---------------------------------------------------------------------------
# the simulation driver (multi_bodies/multi_bodies.py:1112-1627)
def _no_wall(read):
    impl = (read.mobility_blobs_implementation + " " + read.mobility_vector_prod_implementation).lower()
    return read.domain == "no_wall" or "no_wall" in impl


def setup_simulation(read):
    """Bodies, handle and integrator of an input file (read_input.ReadInput):
    structures (vertex + clones files), blob radius, mobility with or without
    the wall, the scheme, forces (gravity and wall repulsion on every blob,
    blob-blob repulsion unless blob_blob_force_implementation is 'None'),
    seed.  Returns (integrator, structures_ID, body_types)."""
    import torch
    from . import clones, forces, integrator
    if read.articulated or len(read.structures) > read.num_free_bodies:
        raise NotImplementedError("articulated bodies and obstacles are not supported")
    if read.body_body_force_torque_implementation != "None":
        raise NotImplementedError("body-body forces are not supported")
    if read.scheme not in integrator.QuaternionIntegrator.SCHEMES:
        raise NotImplementedError("scheme %r is not available on the device" % read.scheme)
    a = read.blob_radius
    r_ref, locs, quats, counts, body_types = [], [], [], [], []
    for files in read.structures:
        if len(files) > 2:
            raise NotImplementedError("slip and Laplace files are not supported")
        ref = clones.read_vertex_file(files[0])
        n, loc, ori = clones.read_clones_file(files[1])
        body_types.append(n)
        for k in range(n):
            r_ref.append(ref)
            counts.append(ref.shape[0])
        locs.append(loc)
        quats.append(ori)
    L = read.periodic_length if read.periodic_length.size == 3 else np.zeros(3)
    system = RigidSystem(counts, read.eta, a, periodic_length=L, wall=not _no_wall(read))
    seed = int(read.seed) if read.seed is not None else int(torch.randint(0, 2 ** 31 - 1, (1,)).item())
    integ = integrator.QuaternionIntegrator(
        system, read.scheme, np.concatenate(locs), np.concatenate(quats), np.concatenate(r_ref),
        tolerance=read.solver_tolerance, domain="no_wall" if _no_wall(read) else "single_wall", kT=read.kT,
        rf_delta=read.rf_delta, mode=read.gb300_precision, seed=seed)
    kw = {"g": read.g, "repulsion_strength_wall": read.repulsion_strength_wall,
          "debye_length_wall": read.debye_length_wall, "periodic_length": L}
    if read.blob_blob_force_implementation != "None":
        kw.update(repulsion_strength=read.repulsion_strength, debye_length=read.debye_length)
    integ.force_torque_calculator = lambda s, r: forces.force_torque_calculator_sort_by_bodies(s, r, **kw)
    return integ, list(read.structures_ID), body_types


def main(argv=None):
    """python -m rigidmultiblobswall_gb300.multi_bodies --input-file data.main"""
    import argparse
    import shutil
    from . import clones
    from .read_input import ReadInput
    parser = argparse.ArgumentParser(description="Run a multi-body simulation and save trajectory.")
    parser.add_argument("--input-file", dest="input_file", type=str, default="data.main")
    parser.add_argument("--print-residual", action="store_true")
    args = parser.parse_args(argv)
    read = ReadInput(args.input_file)
    import os
    out_dir = os.path.dirname(read.output_name)
    if out_dir:
        os.makedirs(out_dir, exist_ok=True)
    shutil.copyfile(args.input_file, read.output_name + ".inputfile")
    integ, ids, body_types = setup_simulation(read)
    with open(read.output_name + ".bodies_info", "w") as f:
        f.write("num_of_body_types  " + str(len(ids)) + "\n")
        f.write("body_names         " + str(ids) + "\n")
        f.write("body_types         " + str(body_types) + "\n")
        f.write("num_bodies         " + str(sum(body_types)) + "\n")
        f.write("num_blobs          " + str(integ.system.n_blobs) + "\n")
    clones.run(integ, read.dt, read.n_steps, n_save=read.n_save, output_name=read.output_name, structures_ID=ids,
               body_types=body_types, save_clones=read.save_clones, initial_step=read.initial_step, verbose=True)
    integ.close()
    return integ


if __name__ == "__main__":
    main()
