"""Generate the golden fixtures in this folder from the reference's own FP64 code.

Runs only where a RigidMultiblobsWall checkout is available, named by the
environment variable RMW_REFERENCE_ROOT; it imports the reference's
Python read-only through ``oracle/ref_shims.py`` (numba source run as plain
Python, no fastmath).  The fixtures it writes are small ``.npz`` files that the
tests load on any machine:

  products.npz   the four wall products (mobility/mobility.py *_numba wrappers)
  nowall.npz     the four free-space products (mobility/mobility.py *_no_wall_*_numba)
  forces.npz     blob-blob and external blob forces (multi_bodies/multi_bodies_functions.py)
                 on seeded blobs: far from the wall, overlapping the wall
                 (damping active), with blobs at exactly r = 2a, and periodic;
                 plus the dense wall mobility (mobility/mobility.py:1018-1116)
  rigid.npz      rigid-body pieces and a full mobility solve through
                 multi_bodies.linear_operator_rigid, build_block_diagonal_preconditioner
                 and general_application_utils.gmres (restart 60, tol 1e-8)
  lanczos.npz    stochastic_forcing_lanczos on a dense wall mobility and on the
                 block-preconditioned operator of build_block_diagonal_preconditioners_det_stoch
  shells.npz     the reference's 12- and 42-blob shell vertex files (geometry inputs)
  quaternion.npz Quaternion.from_rotation, products and rotation matrices
  schemes.npz    two time steps of each GMRES-based time integrator of
                 quaternion_integrator_multi_bodies.py with the normal draws it made
  source_target.npz  products with per-blob radii from sources to targets (wall, free
                 space, free surface) and the single-radius free-surface product
  rollers.npz    rollers at a prescribed angular velocity (velocity-and-torque solve,
                 two forward Euler steps) through QuaternionIntegratorRollers
  clones.npz     read_clones_file / read_vertex_file outputs and the trajectory
                 text of multi_bodies/multi_bodies.py:1428-1457

Usage:  python tests/golden/make_golden.py
"""
import os
import sys
from functools import partial

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "..", "oracle"))
import ref_shims  # noqa: E402

REF = ref_shims.REFERENCE_ROOT


def blobs(rng, n, a, zlo, zhi, box):
    r = np.empty((n, 3))
    r[:, 0:2] = rng.uniform(0, box, (n, 2))
    r[:, 2] = rng.uniform(zlo, zhi, n)
    return r


def make_products():
    mb = ref_shims.load("mobility.mobility")
    fns = {
        "uf": mb.single_wall_mobility_trans_times_force_numba,
        "ut": mb.single_wall_mobility_trans_times_torque_numba,
        "wf": mb.single_wall_mobility_rot_times_force_numba,
        "wt": mb.single_wall_mobility_rot_times_torque_numba,
    }
    out = {}
    cases = [
        # name, seed, n, a, eta, zlo, zhi, box, L
        ("far", 10, 80, 0.5, 1.0, 0.75, 5.0, 32.0, None),
        ("damped", 11, 64, 0.4, 0.7, 0.05, 2.0, 6.0, None),
        ("touching", 12, 48, 0.3, 1.3, 0.35, 1.5, 3.0, None),
        ("periodic", 13, 40, 0.5, 1.0, 0.3, 3.0, 8.0, np.array([8.0, 9.0, 0.0])),
        ("single", 14, 1, 0.5, 1.0, 0.3, 0.4, 1.0, None),
    ]
    for name, seed, n, a, eta, zlo, zhi, box, L in cases:
        rng = np.random.default_rng(seed)
        r = blobs(rng, n, a, zlo, zhi, box)
        if name == "touching" and n >= 4:
            # exact contact pairs at r = 2a (the RPY branch point)
            r[1] = r[0] + np.array([2 * a, 0.0, 0.0])
            r[3] = r[2] + np.array([0.0, 0.0, 2 * a])
        v = rng.standard_normal((n, 3))
        kw = {} if L is None else {"periodic_length": L}
        out[name + "_r"] = r
        out[name + "_v"] = v
        out[name + "_params"] = np.array([a, eta])
        out[name + "_L"] = np.zeros(3) if L is None else L
        for k, fn in fns.items():
            out[name + "_" + k] = fn(r, v, eta, a, **kw)
        if L is None and n <= 64:
            out[name + "_dense"] = mb.single_wall_fluid_mobility(r, eta, a)
    np.savez_compressed(os.path.join(HERE, "products.npz"), **out)


def make_nowall():
    """Free-space products of the reference's no-wall numba functions
    (mobility/mobility.py *_no_wall_*_numba wrappers).  Blobs may sit at any
    height, below z = 0 included: there is no wall and no regularisation."""
    mb = ref_shims.load("mobility.mobility")
    fns = {
        "uf": mb.no_wall_mobility_trans_times_force_numba,
        "ut": mb.no_wall_mobility_trans_times_torque_numba,
        "wf": mb.no_wall_mobility_rot_times_force_numba,
        "wt": mb.no_wall_mobility_rot_times_torque_numba,
    }
    out = {}
    cases = [
        ("far", 20, 80, 0.5, 1.0, -3.0, 5.0, 32.0, None),
        ("touching", 21, 48, 0.3, 1.3, -0.5, 1.5, 3.0, None),
        ("periodic", 22, 40, 0.5, 1.0, -2.0, 3.0, 8.0, np.array([8.0, 9.0, 7.0])),
        ("single", 23, 1, 0.5, 1.0, 0.3, 0.4, 1.0, None),
    ]
    for name, seed, n, a, eta, zlo, zhi, box, L in cases:
        rng = np.random.default_rng(seed)
        r = blobs(rng, n, a, zlo, zhi, box)
        if name == "touching" and n >= 4:
            r[1] = r[0] + np.array([2 * a, 0.0, 0.0])
            r[3] = r[2] + np.array([0.0, 0.0, 2 * a])
        v = rng.standard_normal((n, 3))
        kw = {"periodic_length": np.zeros(3) if L is None else L}
        out[name + "_r"] = r
        out[name + "_v"] = v
        out[name + "_params"] = np.array([a, eta])
        out[name + "_L"] = kw["periodic_length"]
        for k, fn in fns.items():
            out[name + "_" + k] = fn(r, v, eta, a, **kw)
        if L is None:
            # dense free-space blob mobility of the preconditioner (python_no_wall)
            out[name + "_dense"] = mb.rotne_prager_tensor(r, eta, a)
    np.savez_compressed(os.path.join(HERE, "nowall.npz"), **out)


def make_forces():
    """Blob forces of the reference's Python implementations
    (multi_bodies/multi_bodies_functions.py): calc_blob_blob_forces_python
    (soft repulsion, both branches, periodic minimum image), its neighbour-list
    variant calc_blob_blob_forces_tree_numba (multi_bodies/forces_numba.py) and
    blob_external_forces (gravity and wall repulsion, blobs above and below a)."""
    mbf = ref_shims.load_script("multi_bodies/multi_bodies_functions.py", "multi_bodies_functions")
    out = {}
    cases = [
        # name, seed, n, box, zlo, zhi, eps, b, a, L
        ("dense", 30, 60, 3.0, 0.0, 2.0, 1.3, 0.2, 0.3, None),
        ("periodic", 31, 50, 4.0, 0.1, 3.0, 0.7, 0.5, 0.25, np.array([4.0, 4.0, 0.0])),
        ("far", 32, 30, 40.0, 0.5, 9.0, 2.0, 0.1, 0.4, None),
    ]
    for name, seed, n, box, zlo, zhi, eps, b, a, L in cases:
        rng = np.random.default_rng(seed)
        r = blobs(rng, n, a, zlo, zhi, box)
        kw = {"periodic_length": np.zeros(3) if L is None else L, "repulsion_strength": eps, "debye_length": b,
              "blob_radius": a}
        out[name + "_r"] = r
        out[name + "_params"] = np.array([eps, b, a])
        out[name + "_L"] = kw["periodic_length"]
        out[name + "_bb"] = mbf.calc_blob_blob_forces_python(r.copy(), **kw)
        # neighbour-list variant, truncated at 2a + 30 b (multi_bodies/forces_numba.py:228-270)
        import forces_numba
        out[name + "_tree"] = forces_numba.calc_blob_blob_forces_tree_numba(r.copy(), **kw)
        ext = {"blob_mass": 1.7, "blob_radius": a, "g": 0.9, "repulsion_strength_wall": 0.6,
               "debye_length_wall": 0.15}
        out[name + "_ext_params"] = np.array([ext["blob_mass"], ext["blob_radius"], ext["g"],
                                              ext["repulsion_strength_wall"], ext["debye_length_wall"]])
        out[name + "_ext"] = mbf.blob_external_forces(r.copy(), **ext)
    np.savez_compressed(os.path.join(HERE, "forces.npz"), **out)


def read_vertex(rel):
    rv = ref_shims.load("read_input.read_vertex_file")
    return rv.read_vertex_file(os.path.join(REF, rel))


def make_shells():
    s42 = read_vertex("multi_bodies/Structures/shell_N_42_Rg_0_8913_Rh_1.vertex")
    s12 = read_vertex("multi_bodies/Structures/shell_N_12_Rg_1.vertex")
    np.savez_compressed(os.path.join(HERE, "shells.npz"), shell42=s42, shell12=s12)
    return s42, s12


def random_quaternions(rng, n):
    q = rng.standard_normal((n, 4))
    return q / np.linalg.norm(q, axis=1)[:, None]


def make_quaternion():
    Q = ref_shims.load("quaternion_integrator.quaternion").Quaternion
    rng = np.random.default_rng(20)
    q = random_quaternions(rng, 8)
    phi = rng.standard_normal((8, 3)) * 0.3
    phi[0] = 0.0
    rot = np.array([Q(x).rotation_matrix() for x in q])
    fr = np.array([Q.from_rotation(p).entries for p in phi])
    prod = np.array([(Q.from_rotation(p) * Q(x)).entries for p, x in zip(phi, q)])
    np.savez_compressed(os.path.join(HERE, "quaternion.npz"), q=q, phi=phi, rot=rot,
                        from_rotation=fr, product=prod)


def place_bodies(rng, nb, R, a, box, zlo, zhi):
    locs = []
    for _ in range(100000):
        if len(locs) == nb:
            break
        c = np.array([rng.uniform(0, box), rng.uniform(0, box), rng.uniform(zlo, zhi)])
        if all(np.linalg.norm(c - o) > 2 * R + 2 * a for o in locs):
            locs.append(c)
    assert len(locs) == nb, "body placement failed"
    return np.array(locs)


def make_rigid(s42, s12):
    Q = ref_shims.load("quaternion_integrator.quaternion").Quaternion
    body_mod = ref_shims.load("body.body")
    mb = ref_shims.load("mobility.mobility")
    utils = ref_shims.load("general_application_utils")
    mbs = ref_shims.load_script("multi_bodies/multi_bodies.py", "ref_multi_bodies")
    from scipy.spatial.distance import pdist
    out = {}
    for name, ref_cfg, nb, seed, zlo_f, box_f in (("s42", s42, 6, 30, 1.2, 8.0), ("s12", s12, 8, 31, 1.05, 16.0)):
        R = np.linalg.norm(ref_cfg[0])
        a = 0.5 * pdist(ref_cfg).min()
        eta = 1.0
        rng = np.random.default_rng(seed)
        locs = place_bodies(rng, nb, R, a, box_f * R, zlo_f * R, 3 * R)
        quats = random_quaternions(rng, nb)
        bodies = []
        for k in range(nb):
            b = body_mod.Body(locs[k], Q(quats[k]), ref_cfg, a)
            b.mobility_blobs = mb.single_wall_fluid_mobility
            bodies.append(b)
        Nblobs = sum(b.Nblobs for b in bodies)
        r = mbs.get_blobs_r_vectors(bodies, Nblobs)
        mbs.mobility_vector_prod = mb.single_wall_fluid_mobility_product
        K_bodies = mbs.calc_K_matrix_bodies(bodies, Nblobs)
        size = 3 * Nblobs + 6 * nb
        x = rng.standard_normal(size)
        Ax = mbs.linear_operator_rigid(x, bodies, [], r, eta, a, K_bodies=K_bodies, periodic_length=np.zeros(3))
        mbs.build_block_diagonal_preconditioner.mobility_bodies = []
        mbs.build_block_diagonal_preconditioner.initialized = []
        PC = mbs.build_block_diagonal_preconditioner(bodies, [], r, Nblobs, eta, a, periodic_length=np.zeros(3),
                                                     update_PC=1, step=0)
        Px = PC(x)
        # Mobility problem: force (0,0,-1) per body, zero torque, zero slip (cfg-2 style)
        FT = np.zeros((nb, 6))
        FT[:, 2] = -1.0
        FT[:, 3:6] = rng.standard_normal((nb, 3)) * 0.1
        RHS = np.concatenate([np.zeros(3 * Nblobs), -FT.flatten()])
        RHS_norm = np.linalg.norm(RHS)
        import scipy.sparse.linalg as spla
        A = spla.LinearOperator((size, size), matvec=partial(mbs.linear_operator_rigid, bodies=bodies, constraints=[],
                                                             r_vectors=r, eta=eta, a=a, K_bodies=K_bodies,
                                                             periodic_length=np.zeros(3)), dtype="float64")
        P = spla.LinearOperator((size, size), matvec=PC, dtype="float64")
        it = [0]

        def cb(rk):
            it[0] += 1
        sol, info = utils.gmres(A, RHS / RHS_norm, tol=1e-8, M=P, maxiter=1000, restart=60, callback=cb)
        sol = sol * RHS_norm
        true_res = np.linalg.norm(RHS - A.matvec(sol)) / RHS_norm
        # stochastic det/stoch preconditioners and a Lanczos draw through them
        sf = ref_shims.load("stochastic_forcing.stochastic_forcing")
        mbs.build_block_diagonal_preconditioners_det_stoch.mobility_bodies = []
        mbs.build_block_diagonal_preconditioners_det_stoch.initialized = []
        PC2, mob_pc, P_inv = mbs.build_block_diagonal_preconditioners_det_stoch(
            bodies, r, Nblobs, eta, a, periodic_length=np.zeros(3), update_PC=1, step=0)
        w = rng.standard_normal(3 * Nblobs)
        mob_pc_w = mob_pc(w.copy())
        P_inv_w = P_inv(w.copy())
        z = rng.standard_normal(3 * Nblobs)
        noise, lit = sf.stochastic_forcing_lanczos(factor=np.sqrt(2.0 * 1.0 / 1e-3), tolerance=1e-3,
                                                   dim=3 * Nblobs, mobility_mult=mob_pc, L_mult=P_inv, z=z)
        # One Euler-Maruyama step with that noise, as stochastic_EM does
        # (quaternion_integrator_multi_bodies.py:262-322): RHS = [-noise; -FT]
        # scaled to norm 1, GMRES with the deterministic PC, then x += U dt and
        # q <- from_rotation(w dt) * q.
        dt = 1e-3
        RHS2 = np.concatenate([-noise, -FT.flatten()])
        n2 = np.linalg.norm(RHS2)
        sol2, info2 = utils.gmres(A, RHS2 / n2, tol=1e-8, M=spla.LinearOperator((size, size), matvec=PC2,
                                                                                dtype="float64"),
                                  maxiter=1000, restart=60)
        sol2 = sol2 * n2
        vel = sol2[3 * Nblobs:]
        new_locs = np.array([locs[k] + vel[6 * k:6 * k + 3] * dt for k in range(nb)])
        new_quats = np.array([(Q.from_rotation(vel[6 * k + 3:6 * k + 6] * dt) * Q(quats[k])).entries
                              for k in range(nb)])
        p = name + "_"
        out.update({p + "bd_dt": np.array([dt]), p + "bd_sol": sol2, p + "bd_locs": new_locs,
                    p + "bd_quats": new_quats, p + "bd_info": np.array([info2])})
        out.update({p + "ref_cfg": ref_cfg, p + "locs": locs, p + "quats": quats, p + "params": np.array([a, eta]),
                    p + "r": r, p + "K": np.array(K_bodies), p + "x": x, p + "Ax": Ax, p + "Px": Px,
                    p + "FT": FT, p + "sol": sol, p + "info": np.array([info, it[0]]), p + "true_res": np.array([true_res]),
                    p + "w": w, p + "mob_pc_w": mob_pc_w, p + "P_inv_w": P_inv_w, p + "z": z,
                    p + "noise": noise, p + "lanczos_iters": np.array([lit])})
        print(name, "bodies", nb, "blobs", Nblobs, "gmres info", info, "iters", it[0], "true res", true_res,
              "lanczos iters", lit)
    np.savez_compressed(os.path.join(HERE, "rigid.npz"), **out)


def make_lanczos():
    mb = ref_shims.load("mobility.mobility")
    sf = ref_shims.load("stochastic_forcing.stochastic_forcing")
    rng = np.random.default_rng(40)
    out = {}
    for name, n, tol in (("small", 24, 1e-6), ("tight", 40, 1e-10), ("loose", 40, 1e-3)):
        a = 0.5
        r = blobs(rng, n, a, 0.6, 4.0, 8.0)
        M = mb.single_wall_fluid_mobility(r, 1.0, a)
        z = rng.standard_normal(3 * n)
        noise, it = sf.stochastic_forcing_lanczos(factor=1.7, tolerance=tol, mobility=M, z=z)
        out[name + "_r"] = r
        out[name + "_z"] = z
        out[name + "_M"] = M
        out[name + "_tol"] = np.array([tol, 1.7])
        out[name + "_noise"] = noise
        out[name + "_iters"] = np.array([it])
        out[name + "_exact"] = 1.7 * np.real(__import__("scipy").linalg.sqrtm(M)) @ z
    np.savez_compressed(os.path.join(HERE, "lanczos.npz"), **out)


SCHEMES = ("deterministic_forward_euler", "deterministic_adams_bashforth", "deterministic_midpoint",
           "stochastic_EM", "stochastic_first_order_RFD", "stochastic_adams_bashforth", "stochastic_traction_EM",
           "stochastic_traction_AB", "stochastic_Slip_Trapz", "stochastic_Slip_Mid")


def make_schemes(s12):
    """Two time steps of every GMRES-based scheme of the reference's
    QuaternionIntegrator (quaternion_integrator/quaternion_integrator_multi_bodies.py)
    on three 12-blob shells above the wall, wired as multi_bodies/multi_bodies.py:1318-1386
    does (numba wall product, dense wall blocks for the preconditioners, external
    and blob-blob forces of multi_bodies_functions.py), tolerance 1e-12 for GMRES
    and Lanczos.  Every normal draw the schemes make (np.random.normal and the
    np.random.randn of stochastic_forcing_lanczos) is recorded in order, so the
    same draws can be fed to the other implementations."""
    Q = ref_shims.load("quaternion_integrator.quaternion").Quaternion
    qi = ref_shims.load("quaternion_integrator.quaternion_integrator_multi_bodies")
    body_mod = ref_shims.load("body.body")
    mb = ref_shims.load("mobility.mobility")
    mbs = ref_shims.load_script("multi_bodies/multi_bodies.py", "ref_multi_bodies")
    mbf = ref_shims.load_script("multi_bodies/multi_bodies_functions.py", "multi_bodies_functions")
    from scipy.spatial.distance import pdist
    mbf.calc_blob_blob_forces = mbf.calc_blob_blob_forces_python
    mbf.calc_body_body_forces_torques = mbf.set_body_body_forces_torques("None")
    mbs.mobility_vector_prod = mb.single_wall_mobility_trans_times_force_numba
    R = np.linalg.norm(s12[0])
    a = 0.5 * pdist(s12).min()
    eta, kT, dt, nb = 1.0, 0.7, 0.02, 3
    L = np.zeros(3)
    fkw = {"g": 1.0, "repulsion_strength_wall": 0.5, "debye_length_wall": 0.1 * a, "repulsion_strength": 0.5,
           "debye_length": 0.1 * a, "periodic_length": L}
    rng = np.random.default_rng(50)
    locs = place_bodies(rng, nb, R, a, 5 * R, 1.6 * R, 2.6 * R)
    quats = random_quaternions(rng, nb)
    out = {"ref_cfg": s12, "locs": locs, "quats": quats,
           "params": np.array([eta, a, kT, dt, 1e-3, 1e-12]),
           "force_params": np.array([1.0, fkw["g"], fkw["repulsion_strength_wall"], fkw["debye_length_wall"],
                                     fkw["repulsion_strength"], fkw["debye_length"]])}
    orig_normal, orig_randn = np.random.normal, np.random.randn
    try:
        for si, scheme in enumerate(SCHEMES):
            bodies = []
            for k in range(nb):
                b = body_mod.Body(locs[k].copy(), Q(quats[k].copy()), s12, a)
                b.mobility_blobs = mb.single_wall_fluid_mobility
                if k == 0:
                    b.calc_body_length()
                else:
                    b.body_length = bodies[0].body_length
                bodies.append(b)
            Nblobs = sum(b.Nblobs for b in bodies)
            integ = qi.QuaternionIntegrator(bodies, Nblobs, scheme, tolerance=1e-12, domain="single_wall")
            integ.build_block_diagonal_preconditioner = mbs.build_block_diagonal_preconditioner
            integ.first_guess = np.zeros(3 * Nblobs + 6 * nb)
            integ.calc_slip = None
            integ.get_blobs_r_vectors = mbs.get_blobs_r_vectors
            integ.mobility_blobs = mb.single_wall_fluid_mobility
            integ.mobility_vector_prod = mb.single_wall_mobility_trans_times_force_numba
            integ.force_torque_calculator = partial(mbf.force_torque_calculator_sort_by_bodies, **fkw)
            integ.calc_K_matrix_bodies = mbs.calc_K_matrix_bodies
            integ.calc_K_matrix = mbs.calc_K_matrix
            integ.linear_operator = mbs.linear_operator_rigid
            integ.build_block_diagonal_preconditioners_det_stoch = mbs.build_block_diagonal_preconditioners_det_stoch
            integ.eta, integ.a, integ.kT = eta, a, kT
            integ.K_matrix_T_vector_prod = mbs.K_matrix_T_vector_prod
            integ.K_matrix_vector_prod = mbs.K_matrix_vector_prod
            integ.preprocess = mbf.preprocess
            integ.postprocess = mbf.postprocess
            integ.periodic_length = L
            integ.update_PC = 1
            integ.print_residual = False
            integ.rf_delta = 1e-3
            integ.constraints = []
            integ.articulated = []
            for f in (mbs.build_block_diagonal_preconditioner, mbs.build_block_diagonal_preconditioners_det_stoch):
                f.mobility_bodies = []
                f.initialized = []
            rs = np.random.RandomState(60 + si)
            draws = []

            def normal(loc=0.0, scale=1.0, size=None):
                assert loc == 0.0 and scale == 1.0
                x = rs.normal(loc, scale, size)
                draws.append(np.array(x, dtype=np.float64).ravel().copy())
                return x

            def randn(*shape):
                x = rs.randn(*shape)
                draws.append(np.array(x, dtype=np.float64).ravel().copy())
                return x

            np.random.normal, np.random.randn = normal, randn
            p = scheme + "_"
            for step in range(2):
                integ.advance_time_step(dt, step=step)
                out[p + "locs%d" % step] = np.array([b.location for b in bodies])
                out[p + "quats%d" % step] = np.array([b.orientation.entries for b in bodies])
            np.random.normal, np.random.randn = orig_normal, orig_randn
            out[p + "draws"] = np.concatenate(draws) if draws else np.zeros(0)
            out[p + "draw_sizes"] = np.array([d.size for d in draws])
            out[p + "counts"] = np.array([integ.invalid_configuration_count, integ.det_iterations_count,
                                          integ.stoch_iterations_count])
            out["body_length"] = np.array([bodies[0].body_length])
            print(scheme, "draws", [d.size for d in draws], "counts", out[p + "counts"],
                  "displacement", np.linalg.norm(out[p + "locs1"] - locs, axis=1).max())
    finally:
        np.random.normal, np.random.randn = orig_normal, orig_randn
    np.savez_compressed(os.path.join(HERE, "schemes.npz"), **out)


def make_source_target():
    """Source-target products with per-blob radii (mobility/mobility.py:551-616, 1409-1429 over
    mobility/mobility_numba.py:1480-1660, 1941-2093): wall (shifted heights and damping of
    both sides), free space and free surface; and the single-radius free-surface product
    (mobility.py:1390-1406, mobility_numba.py:1770-1938).  Cases: far pairs; close pairs
    (r < a + b, one blob inside another, a target on a source, blobs below their radius);
    pseudo-periodic in x and y."""
    mb = ref_shims.load("mobility.mobility")
    out = {}
    cases = [
        # name, seed, ns, nt, box, zlo, zhi, rlo, rhi, L
        ("far", 80, 40, 30, 10.0, 0.7, 4.0, 0.2, 0.6, None),
        ("close", 81, 36, 28, 1.6, 0.05, 1.5, 0.1, 0.7, None),
        ("periodic", 82, 30, 24, 5.0, 0.3, 2.5, 0.2, 0.5, np.array([5.0, 6.0, 0.0])),
    ]
    for name, seed, ns, nt, box, zlo, zhi, rlo, rhi, L in cases:
        rng = np.random.default_rng(seed)
        src = blobs(rng, ns, 0.0, zlo, zhi, box)
        trg = blobs(rng, nt, 0.0, zlo, zhi, box)
        rs = rng.uniform(rlo, rhi, ns)
        rt = rng.uniform(rlo, rhi, nt)
        if name == "close":
            trg[0] = src[0]                       # a target on a source (r = 0)
            trg[1] = src[1] + np.array([0.05, 0.0, 0.0])
            rt[1], rs[1] = 0.6, 0.2               # r < |b - a|: one blob inside the other
            trg[2] = src[2] + np.array([0.0, 0.0, rs[2] + rt[2]])   # r = a + b exactly
        f = rng.standard_normal((ns, 3))
        kw = {"periodic_length": np.zeros(3) if L is None else L}
        eta = 0.9
        out[name + "_source"], out[name + "_target"] = src, trg
        out[name + "_rs"], out[name + "_rt"], out[name + "_f"] = rs, rt, f
        out[name + "_L"], out[name + "_eta"] = kw["periodic_length"], np.array([eta])
        out[name + "_wall"] = mb.single_wall_mobility_trans_times_force_source_target_numba(
            src, trg, f, rs, rt, eta, **kw)
        out[name + "_nowall"] = mb.no_wall_mobility_trans_times_force_source_target_numba(
            src, trg, f, rs, rt, eta, **kw)
        out[name + "_free_surface"] = mb.free_surface_mobility_trans_times_force_source_target_numba(
            src, trg, f, rs, rt, eta, **kw)
        if L is None:
            # the Python forms (no periodic images), mobility/mobility.py:830-946
            out[name + "_one_wall_py"] = np.asarray(mb.mobility_vector_product_source_target_one_wall(
                src, trg, f, rs, rt, eta)).reshape(-1)
            out[name + "_unbounded_py"] = np.asarray(mb.mobility_vector_product_source_target_unbounded(
                src, trg, f, rs, rt, eta)).reshape(-1)
    for name, seed, n, a, box, zlo, zhi, L in (("fs", 83, 50, 0.4, 4.0, 0.1, 3.0, None),
                                             ("fs_periodic", 84, 40, 0.5, 4.0, 0.3, 3.0,
                                              np.array([4.0, 5.0, 0.0]))):
        rng = np.random.default_rng(seed)
        r = blobs(rng, n, a, zlo, zhi, box)
        f = rng.standard_normal((n, 3))
        kw = {"periodic_length": np.zeros(3) if L is None else L}
        out[name + "_r"], out[name + "_f"], out[name + "_params"] = r, f, np.array([a, 1.1])
        out[name + "_L"] = kw["periodic_length"]
        out[name + "_u"] = mb.free_surface_mobility_trans_times_force_numba(r, f, 1.1, a, **kw)
    np.savez_compressed(os.path.join(HERE, "source_target.npz"), **out)


def make_rollers():
    """Rollers at a prescribed angular velocity through the reference's
    QuaternionIntegratorRollers (quaternion_integrator/quaternion_integrator_rollers.py):
    compute_deterministic_velocity_and_torque (:905-983) and two
    deterministic_forward_euler steps (:119-152) with the numba wall products,
    gravity, wall and blob-blob repulsion (multi_bodies_functions.py), GMRES
    tolerance 1e-12; prescribed and free kinematics; and free space."""
    qr = ref_shims.load("quaternion_integrator.quaternion_integrator_rollers")
    mbf = ref_shims.load_script("multi_bodies/multi_bodies_functions.py", "multi_bodies_functions")
    mbf.calc_blob_blob_forces = mbf.calc_blob_blob_forces_python
    out = {}
    for name, seed, n, a, domain, free, L in (("wall", 90, 40, 0.5, "single_wall", "False", np.zeros(3)),
                                           ("wall_free", 91, 30, 0.5, "single_wall", "True", np.zeros(3)),
                                           ("periodic", 92, 30, 0.4, "single_wall", "False",
                                            np.array([6.0, 6.0, 0.0])),
                                           ("no_wall", 93, 30, 0.5, "no_wall", "False", np.zeros(3))):
        rng = np.random.default_rng(seed)
        r = blobs(rng, n, a, 1.05 * a, 3.0, 6.0)
        fkw = {"g": 0.8, "repulsion_strength_wall": 0.4, "debye_length_wall": 0.2 * a}
        bkw = dict(fkw, repulsion_strength=0.6, debye_length=0.2 * a, periodic_length=L)

        class Blob:
            def __init__(self, x):
                self.location = np.array(x)

        bodies = [Blob(x) for x in r]
        integ = qr.QuaternionIntegratorRollers(bodies, n, "deterministic_forward_euler_rollers", tolerance=1e-12,
                                               domain=domain, mobility_vector_prod_implementation="numba")
        integ.calc_one_blob_forces = partial(mbf.calc_one_blob_forces, **fkw)
        integ.calc_blob_blob_forces = partial(mbf.calc_blob_blob_forces, **bkw)
        integ.eta, integ.a = 0.9, a
        integ.omega_one_roller = np.array([0.0, 2.0, 0.3])
        integ.free_kinematics = free
        integ.hydro_interactions = 1
        integ.periodic_length = L
        integ.print_residual = False
        force = np.asarray(mbf.calc_one_blob_forces(r.copy(), blob_radius=a, blob_mass=1.0, **fkw)).reshape(-1) + \
            np.asarray(mbf.calc_blob_blob_forces(r.copy(), blob_radius=a, **bkw)).reshape(-1)
        u, t = integ.compute_deterministic_velocity_and_torque()
        p = name + "_"
        out.update({p + "r": r, p + "force": force, p + "params": np.array([0.9, a]), p + "omega": integ.omega_one_roller,
                    p + "L": L, p + "velocity": np.asarray(u).reshape(-1), p + "torque": np.asarray(t).reshape(-1),
                    p + "force_params": np.array([fkw["g"], fkw["repulsion_strength_wall"], fkw["debye_length_wall"],
                                                  bkw["repulsion_strength"], bkw["debye_length"]])})
        integ.deterministic_torque_previous_step = None
        for step in range(2):
            integ.advance_time_step(0.01)
            out[p + "x%d" % step] = np.array([b.location for b in bodies])
    np.savez_compressed(os.path.join(HERE, "rollers.npz"), **out)


def make_clones():
    """Structure-file reading and trajectory text of the reference:
    read_clones_file / read_vertex_file (read_input/) on two of the reference's
    structure files and on a synthetic clones text (comments, blank lines,
    unnormalised quaternions, lines past the last body), and the body lines
    that multi_bodies/multi_bodies.py:1428-1457 writes ('%s' of numpy float64
    locations and Quaternion.entries)."""
    import tempfile
    Q = ref_shims.load("quaternion_integrator.quaternion").Quaternion
    rc = ref_shims.load("read_input.read_clones_file")
    rv = ref_shims.load("read_input.read_vertex_file")
    out = {}
    for key, rel in (("shell12", "multi_bodies/Structures/shell_N_12_Rg_1"),
                     ("boomerang15", "multi_bodies/Structures/boomerang_N_15")):
        with open(os.path.join(REF, rel + ".clones")) as f:
            out[key + "_clones_text"] = np.array(f.read())
        n, loc, ori = rc.read_clones_file(os.path.join(REF, rel + ".clones"))
        out[key + "_n"] = np.array([n])
        out[key + "_locations"] = np.asarray(loc, dtype=np.float64).reshape(-1, 3)
        out[key + "_orientations"] = np.array([q.entries for q in ori]).reshape(-1, 4)
        with open(os.path.join(REF, rel + ".vertex")) as f:
            out[key + "_vertex_text"] = np.array(f.read())
        out[key + "_vertex"] = rv.read_vertex_file(os.path.join(REF, rel + ".vertex"))
    synthetic = ("# header comment\n\n   3   # three bodies\n"
                 "0.5 1.5 2.5 2.0 0.0 0.0 0.0\n"
                 "\n# a comment line between bodies\n"
                 "-1e-3 7 1.25e2   0.3 -0.4 0.5 0.6  # trailing comment\n"
                 "4 5 6 1 1 1 1 extra tokens\n"
                 "9 9 9 1 0 0 0\n")
    out["synthetic_clones_text"] = np.array(synthetic)
    with tempfile.TemporaryDirectory() as d:
        p = os.path.join(d, "s.clones")
        with open(p, "w") as f:
            f.write(synthetic)
        n, loc, ori = rc.read_clones_file(p)
    out["synthetic_n"] = np.array([n])
    out["synthetic_locations"] = np.asarray(loc, dtype=np.float64)
    out["synthetic_orientations"] = np.array([q.entries for q in ori])
    rng = np.random.default_rng(70)
    locs = rng.standard_normal((5, 3)) * np.array([1.0, 1e-7, 3e5])
    locs[0] = [0.1, -0.0, 1e17]
    quats = random_quaternions(rng, 5)
    text = str(locs.shape[0]) + "\n"
    for k in range(locs.shape[0]):
        location = locs[k]
        orientation = Q(quats[k]).entries
        text += "%s %s %s %s %s %s %s\n" % (location[0], location[1], location[2], orientation[0], orientation[1],
                                            orientation[2], orientation[3])
    out["write_locations"] = locs
    out["write_orientations"] = quats
    out["write_text"] = np.array(text)
    # input files through the reference's ReadInput (read_input/read_input.py)
    ri = ref_shims.load("read_input.read_input")
    inp = ("# comment line\nscheme   stochastic_Slip_Trapz  # trailing\n\ndt 0.005\nn_steps 20\nn_save 5\n"
           "eta 0.8\ng 1.5\nblob_radius 0.25\nkT 0.3\nsolver_tolerance 1e-9\nrf_delta 2e-3\n"
           "periodic_length 10 12 0\nmobility_vector_prod_implementation numba_no_wall\n"
           "blob_blob_force_implementation python\nrepulsion_strength 2.5\ndebye_length 0.1\n"
           "output_name out/run\nsave_clones one_file\nseed 7\n"
           # given explicitly: the reference parses their 'None' defaults with np.fromstring,
           # which numpy 2 rejects
           "plot_velocity_field 0 1 2\nplot_concentration_field 0 1 2\nbackground_Laplace 0 0 0\n"
           "structure Structures/shell_N_12_Rg_1.vertex Structures/shell_N_12_Rg_1.clones\n"
           "structure Structures/boomerang_N_15.vertex Structures/boomerang_N_15.clones\n")
    keys = ["n_steps", "initial_step", "n_save", "dt", "eta", "g", "blob_radius", "kT", "scheme", "output_name",
            "repulsion_strength_wall", "debye_length_wall", "mobility_blobs_implementation",
            "mobility_vector_prod_implementation", "repulsion_strength", "debye_length",
            "blob_blob_force_implementation", "solver_tolerance", "rf_delta", "save_clones", "domain", "update_PC",
            "hydro_interactions", "seed"]
    with tempfile.TemporaryDirectory() as d:
        for tag, extra in (("input", ""), ("restart", "initial_step 10\n")):
            p = os.path.join(d, tag + ".dat")
            with open(p, "w") as f:
                f.write(inp + extra)
            rd = ri.ReadInput(p)
            out[tag + "_text"] = np.array(inp + extra)
            out[tag + "_values"] = np.array([str(getattr(rd, k)) for k in keys])
            out[tag + "_periodic_length"] = np.asarray(rd.periodic_length, dtype=np.float64)
            out[tag + "_structures"] = np.array([" ".join(s) for s in rd.structures])
            out[tag + "_structures_ID"] = np.array(rd.structures_ID)
    out["input_keys"] = np.array(keys)
    np.savez_compressed(os.path.join(HERE, "clones.npz"), **out)


if __name__ == "__main__":
    # optional arguments select fixture sets (e.g. "nowall"); default: all
    want = set(sys.argv[1:])
    if not want or "products" in want:
        make_products()
    if not want or "nowall" in want:
        make_nowall()
    if not want or "forces" in want:
        make_forces()
    if not want or want & {"shells", "rigid", "schemes"}:
        s42, s12 = make_shells()
    if not want or "quaternion" in want:
        make_quaternion()
    if not want or "rigid" in want:
        make_rigid(s42, s12)
    if not want or "lanczos" in want:
        make_lanczos()
    if not want or "schemes" in want:
        make_schemes(s12)
    if not want or "clones" in want:
        make_clones()
    if not want or "source_target" in want:
        make_source_target()
    if not want or "rollers" in want:
        make_rollers()
    print("golden fixtures written to", HERE)
