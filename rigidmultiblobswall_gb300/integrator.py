"""Rigid-body mobility problem and one Brownian-dynamics Euler-Maruyama step on
the GPU, following quaternion_integrator/quaternion_integrator_multi_bodies.py:
solve_mobility_problem (1441-1547) and stochastic_EM (262-322).

State lives on the device: body locations x (Nb,3), quaternions q (Nb,4),
body-frame blob coordinates r_ref (N,3), body forces/torques FT (Nb,6).
"""
import math

from .rigid import RigidSystem


def mobility_rhs(sys_, force_torque, slip=None, noise=None):
    """RHS = [slip - noise; -F/T] (quaternion_integrator_multi_bodies.py:1476-1489)."""
    import torch
    n3 = 3 * sys_.n_blobs
    dev = sys_.device
    rhs = torch.empty(sys_.size, dtype=torch.float64, device=dev)
    top = rhs[:n3]
    as_dev = lambda v: torch.as_tensor(v, dtype=torch.float64, device=dev).reshape(-1)
    if slip is None and noise is None:
        top.zero_()
    elif noise is None:
        top.copy_(as_dev(slip))
    elif slip is None:
        torch.neg(as_dev(noise), out=top)
    else:
        torch.sub(as_dev(slip), as_dev(noise), out=top)
    torch.neg(as_dev(force_torque), out=rhs[n3:])
    return rhs


def solve_mobility_problem(sys_, force_torque, slip=None, noise=None, tol=1e-8, restart=60, maxiter=1000,
                           mode="fp64"):
    """Solution [lambda; U] of the mobility problem.  The RHS is scaled to norm 1
    before GMRES and the solution scaled back, as the reference does.
    Returns (solution, info, iterations, relative residual)."""
    import numpy as np
    host = all(x is None or isinstance(x, (np.ndarray, list, tuple)) for x in (force_torque, slip, noise))
    if host:
        # host inputs: the scaled RHS is formed on the host and copied once (no device round trip for |b|)
        n3 = 3 * sys_.n_blobs
        rhs = np.zeros(sys_.size)
        if slip is not None:
            rhs[:n3] = np.asarray(slip, dtype=np.float64).reshape(-1)
        if noise is not None:
            rhs[:n3] -= np.asarray(noise, dtype=np.float64).reshape(-1)
        rhs[n3:] = -np.asarray(force_torque, dtype=np.float64).reshape(-1)
        nrm = float(np.linalg.norm(rhs))
        if nrm == 0.0:
            import torch
            return torch.zeros(sys_.size, dtype=torch.float64, device=sys_.device), 0, 0, 0.0
        sol, info, its, rr = sys_.solve(rhs / nrm, tol=tol, restart=restart, maxiter=maxiter, mode=mode)
        return sol.mul_(nrm), info, its, rr
    # device inputs: |b|, the scaling and the scaling back run in the library (one synchronisation)
    rhs = mobility_rhs(sys_, force_torque, slip, noise)
    return sys_.solve(rhs, tol=tol, restart=restart, maxiter=maxiter, mode=mode, scaled=True)


class BrownianStepper:
    """stochastic_EM on the GPU for one suspension of rigid bodies.

    step() builds the stochastic block-diagonal preconditioner, draws the
    Brownian noise sqrt(2 kT / dt) M^(1/2) W by preconditioned Lanczos, solves
    the mobility problem with that slip noise, updates locations and
    quaternions and rejects the step (redraws the noise) if a blob crossed the
    wall, like the reference's check_positions.

    nearfield: None, or (model, exact_cutoff) to augment every step's
    block-diagonal preconditioner (nearfield.NearfieldModel or None for exact
    near-field couplings only).  A step whose augmented solve does not reach
    the tolerance is solved again with the plain preconditioner.
    """

    def __init__(self, sys_: RigidSystem, x, q, r_ref, kT=1.0, lanczos_tol=1e-3, gmres_tol=1e-8, mode="fp64",
                 seed=0, nearfield=None):
        import torch
        self.sys = sys_
        dev = sys_.device
        self.x = torch.as_tensor(x, dtype=torch.float64, device=dev).reshape(-1, 3).clone()
        self.q = torch.as_tensor(q, dtype=torch.float64, device=dev).reshape(-1, 4).clone()
        self.r_ref = torch.as_tensor(r_ref, dtype=torch.float64, device=dev).reshape(-1, 3).contiguous()
        self.kT = kT
        self.lanczos_tol = lanczos_tol
        self.gmres_tol = gmres_tol
        self.mode = mode
        self.gen = torch.Generator(device=dev)
        self.gen.manual_seed(seed)
        self.invalid = 0
        self.lanczos_iterations = 0
        self.gmres_iterations = 0
        self.nearfield = nearfield
        self.fallbacks = 0

    def r_vectors(self):
        return self.sys.blob_positions(self.x, self.q, self.r_ref)

    def step(self, dt, force_torque, z=None, max_retries=100):
        import torch
        s = self.sys
        for _ in range(max_retries):
            r = self.r_vectors()
            s.set_configuration(r, self.x)
            s.build_pc(stochastic=True, mode=self.mode)
            zz = z if z is not None else torch.randn(3 * s.n_blobs, generator=self.gen, dtype=torch.float64,
                                                     device=s.device)
            noise, it_l = s.lanczos(zz, factor=math.sqrt(2.0 * self.kT / dt), tol=self.lanczos_tol,
                                    mode=self.mode)
            self.lanczos_iterations += it_l
            if self.nearfield is not None:
                from . import nearfield as nf
                model, cut = self.nearfield
                if model is None:
                    nf.attach_exact(s, cut)
                else:
                    model.attach(s, cut)
            sol, info, its, rr = solve_mobility_problem(s, force_torque, noise=noise, tol=self.gmres_tol,
                                                        mode=self.mode)
            if self.nearfield is not None and (info != 0 or not rr <= self.gmres_tol):
                from . import nearfield as nf
                nf.detach(s)
                self.fallbacks += 1
                self.gmres_iterations += its
                sol, info, its, rr = solve_mobility_problem(s, force_torque, noise=noise, tol=self.gmres_tol,
                                                            mode=self.mode)
            self.gmres_iterations += its
            vel = sol[3 * s.n_blobs:]
            xn, qn = s.euler_update(self.x, self.q, vel, dt)
            rn = s.blob_positions(xn, qn, self.r_ref)
            if s.count_below(rn, 0.0) == 0:
                self.x, self.q = xn, qn
                return {"velocities": vel, "noise": noise, "lanczos_iterations": it_l, "gmres_iterations": its,
                        "gmres_info": info, "relres": rr}
            self.invalid += 1
            z = None  # a rejected step redraws the noise
        raise RuntimeError("Brownian step rejected %d times in a row" % max_retries)


def body_lengths(blobs_per_body, r_ref, a):
    """Per body: the largest distance between two of its reference blobs plus
    2a; 10 for bodies of more than 2000 blobs (body/body.py:218-231 and its use
    in multi_bodies/multi_bodies.py:1196-1202).  Bodies of equal blob count are
    evaluated together on the device."""
    import numpy as np
    import torch
    counts = np.asarray(blobs_per_body, dtype=np.int64)
    off = np.concatenate([[0], np.cumsum(counts)])
    out = torch.empty(counts.size, dtype=torch.float64, device=r_ref.device)
    for nb in np.unique(counts):
        idx = np.nonzero(counts == nb)[0]
        if nb > 2000:
            out[torch.as_tensor(idx, device=out.device)] = 10.0
            continue
        rows = (off[idx][:, None] + np.arange(nb)[None, :]).reshape(-1)
        blk = r_ref[torch.as_tensor(rows, device=r_ref.device)].reshape(idx.size, nb, 3)
        dmax = torch.cdist(blk, blk).flatten(1).max(dim=1).values
        out[torch.as_tensor(idx, device=out.device)] = dmax + 2.0 * a
    return out


class QuaternionIntegrator:
    """The GMRES-based time integrators of
    quaternion_integrator/quaternion_integrator_multi_bodies.py on the device,
    for one suspension of rigid bodies above a wall (or in free space).

    scheme: deterministic_forward_euler (:75), deterministic_adams_bashforth
    (:142), deterministic_midpoint (:188), stochastic_EM (:262),
    stochastic_first_order_RFD (:326), stochastic_adams_bashforth (:431),
    stochastic_traction_EM (:626), stochastic_traction_AB (:803),
    stochastic_Slip_Trapz (:925) or stochastic_Slip_Mid (:1214);
    advance_time_step(dt) runs it.  Attributes as the reference's: kT,
    tolerance (GMRES and Lanczos), rf_delta, domain ('single_wall' rejects and
    redraws steps that put a blob below z = 0), force_torque_calculator
    (callable(system, r_vectors) -> body forces-torques [F_1, T_1, ...] of
    shape (2 Nb, 3) on the device; None = zero), calc_slip (callable(system,
    r_vectors) -> (N, 3) slip; None = zero), preprocess / postprocess hooks,
    the iteration and invalid-configuration counters, first_step and
    velocities_previous_step.

    State on the device: locations x (Nb,3), quaternions q (Nb,4), body-frame
    blob coordinates r_ref (N,3).  normal(n) supplies the standard normal
    draws, in the reference's order; by default a seeded torch generator.

    The step's configuration lives in `system` (its stochastic preconditioner
    serves the Lanczos noise and the solves there); displaced configurations
    (the random finite differences and the predictor of the two-stage
    schemes) use a second handle of the same bodies, so the first keeps its
    factorisations for the rest of the step.  GMRES starts from zero and every
    configuration solves with its own block-diagonal preconditioner; neither
    changes a result beyond the tolerance (the reference warm-starts and reuses
    the step's preconditioner).  Bodies with prescribed kinematics and
    constraints are not part of this path.
    """

    SCHEMES = ("deterministic_forward_euler", "deterministic_adams_bashforth", "deterministic_midpoint",
               "stochastic_EM", "stochastic_first_order_RFD", "stochastic_adams_bashforth",
               "stochastic_traction_EM", "stochastic_traction_AB", "stochastic_Slip_Trapz", "stochastic_Slip_Mid")

    def __init__(self, system: RigidSystem, scheme, x, q, r_ref, tolerance=1e-8, domain="single_wall", kT=0.0,
                 rf_delta=1e-3, mode="fp64", body_length=None, normal=None, seed=0, restart=60, maxiter=1000):
        import torch
        if scheme not in self.SCHEMES:
            raise ValueError("unknown scheme %r (available: %s)" % (scheme, ", ".join(self.SCHEMES)))
        self.system = system
        dev = system.device
        self.scheme = scheme
        self.x = torch.as_tensor(x, dtype=torch.float64, device=dev).reshape(-1, 3).clone()
        self.q = torch.as_tensor(q, dtype=torch.float64, device=dev).reshape(-1, 4).clone()
        self.r_ref = torch.as_tensor(r_ref, dtype=torch.float64, device=dev).reshape(-1, 3).contiguous()
        if self.x.shape[0] != system.n_bodies or self.q.shape[0] != system.n_bodies \
                or self.r_ref.shape[0] != system.n_blobs:
            raise ValueError("state sizes do not match the suspension")
        self.tolerance = tolerance
        self.domain = domain
        self.kT = kT
        self.rf_delta = rf_delta
        self.mode = mode
        self.restart, self.maxiter = restart, maxiter
        if body_length is None:
            self.body_length = body_lengths(system.blobs_per_body, self.r_ref, system.a)
        else:
            self.body_length = torch.as_tensor(body_length, dtype=torch.float64, device=dev).expand(
                system.n_bodies).contiguous()
        if normal is None:
            gen = torch.Generator(device=dev)
            gen.manual_seed(seed)
            normal = lambda n: torch.randn(n, generator=gen, dtype=torch.float64, device=dev)  # noqa: E731
        self.normal = normal
        self.force_torque_calculator = None
        self.calc_slip = None
        self.preprocess = None
        self.postprocess = None
        self.first_step = True
        self.velocities_previous_step = None
        self.velocities = None
        self.invalid_configuration_count = 0
        self.det_iterations_count = 0
        self.stoch_iterations_count = 0
        self._aux = None

    # -- configuration ---------------------------------------------------------
    @property
    def aux(self):
        if self._aux is None:
            s = self.system
            self._aux = RigidSystem(s.blobs_per_body, s.eta, s.a, periodic_length=s.L, device=s.device, wall=s.wall)
        return self._aux

    def get_blobs_r_vectors(self, x=None, q=None):
        return self.system.blob_positions(self.x if x is None else x, self.q if q is None else q, self.r_ref)

    def _at(self, S, x, q, stochastic=False):
        """Put the bodies of handle S at (x, q); stochastic builds the
        factorisations the Lanczos noise needs."""
        S.set_configuration(S.blob_positions(x, q, self.r_ref), x)
        if stochastic:
            S.build_pc(stochastic=True, mode=self.mode)
        return S

    def _move(self, x, q, vel, scale, length_scaled=False):
        """location + v scale (translation times body_length if length_scaled),
        from_rotation(w scale) * orientation."""
        v = vel.reshape(-1, 6)
        if length_scaled:
            v = v.clone()
            v[:, :3] *= self.body_length[:, None]
        return self.system.euler_update(x, q, v.reshape(-1), scale)

    def _valid(self, x, q):
        """check_positions (quaternion_integrator_multi_bodies.py:1779-1824):
        with a single wall, no blob below z = 0 (body/body.py:118-139)."""
        if self.domain != "single_wall":
            return True
        if self.system.count_below(self.get_blobs_r_vectors(x, q), 0.0) == 0:
            return True
        self.invalid_configuration_count += 1
        return False

    # -- pieces ----------------------------------------------------------------
    def _force_torque(self, S):
        import torch
        if self.force_torque_calculator is None:
            return torch.zeros(6 * S.n_bodies, dtype=torch.float64, device=S.device)
        ft = self.force_torque_calculator(S, S._r)
        return torch.as_tensor(ft, dtype=torch.float64, device=S.device).reshape(-1)

    def _solve(self, S, RHS=None, noise=None, noise_FT=None):
        """solve_mobility_problem (quaternion_integrator_multi_bodies.py:1441-1547):
        RHS = [slip - noise; -(FT + noise_FT)] unless given, scaled to norm 1."""
        import torch
        n3 = 3 * S.n_blobs
        if RHS is None:
            RHS = torch.zeros(S.size, dtype=torch.float64, device=S.device)
            if self.calc_slip is not None:
                RHS[:n3] = torch.as_tensor(self.calc_slip(S, S._r), dtype=torch.float64,
                                           device=S.device).reshape(-1)
            FT = self._force_torque(S)
            if noise_FT is not None:
                FT = FT + noise_FT
            RHS[n3:] = -FT
        else:
            RHS = RHS.clone()
        if noise is not None:
            RHS[:n3] -= noise
        # the library scales to norm 1 and back (a zero RHS gives a zero solution)
        sol, _, its, _ = S.solve(RHS, tol=self.tolerance, restart=self.restart, maxiter=self.maxiter,
                                 mode=self.mode, scaled=True)
        self.det_iterations_count += its
        return sol

    def _lanczos(self, S, factor, z=None):
        """stochastic_forcing_lanczos with the block-diagonal factors of S
        (stochastic/stochastic_forcing.py:112-264); factor 0 draws nothing."""
        import torch
        if factor == 0.0:
            return torch.zeros(3 * S.n_blobs, dtype=torch.float64, device=S.device)
        if z is None:
            z = self.normal(3 * S.n_blobs)
        noise, it = S.lanczos(z, factor=factor, tol=self.tolerance, mode=self.mode)
        self.stoch_iterations_count += it
        return noise

    def _vel(self, sol):
        return sol[3 * self.system.n_blobs:]

    def _zeros(self, n):
        import torch
        return torch.zeros(n, dtype=torch.float64, device=self.system.device)

    def advance_time_step(self, dt, *args, max_retries=10000, **kwargs):
        """One step of the scheme; rejected configurations are redrawn, as the
        reference's schemes loop until check_positions succeeds (here at most
        max_retries times, then RuntimeError)."""
        step = getattr(self, self.scheme)
        for _ in range(max_retries):
            if self.preprocess is not None:
                self.preprocess(self)
            res = step(dt)
            if res is None:
                continue
            if self.postprocess is not None:
                self.postprocess(self)
            self.x, self.q = res
            return
        raise RuntimeError("%s: step rejected %d times in a row" % (self.scheme, max_retries))

    # -- schemes: each returns the accepted (x, q) or None to redraw ------------
    def deterministic_forward_euler(self, dt):
        S = self._at(self.system, self.x, self.q)
        self.velocities = self._vel(self._solve(S))
        xn, qn = self._move(self.x, self.q, self.velocities, dt)
        return (xn, qn) if self._valid(xn, qn) else None

    def deterministic_adams_bashforth(self, dt):
        S = self._at(self.system, self.x, self.q)
        v = self._vel(self._solve(S))
        va = v if self.first_step else 1.5 * v - 0.5 * self.velocities_previous_step
        xn, qn = self._move(self.x, self.q, va, dt)
        if not self._valid(xn, qn):
            return None
        self.first_step = False
        self.velocities_previous_step = v
        return xn, qn

    def deterministic_midpoint(self, dt):
        x0, q0 = self.x, self.q
        v = self._vel(self._solve(self._at(self.system, x0, q0)))
        xm, qm = self._move(x0, q0, v, 0.5 * dt)
        if not self._valid(xm, qm):
            return None
        vm = self._vel(self._solve(self._at(self.aux, xm, qm)))
        xn, qn = self._move(x0, q0, vm, dt)
        return (xn, qn) if self._valid(xn, qn) else None

    def stochastic_EM(self, dt):
        S = self._at(self.system, self.x, self.q, stochastic=True)
        noise = self._lanczos(S, math.sqrt(2.0 * self.kT / dt))
        xn, qn = self._move(self.x, self.q, self._vel(self._solve(S, noise=noise)), dt)
        return (xn, qn) if self._valid(xn, qn) else None

    def _rfd_drift(self, x0, q0, rfd):
        """Two-solve random finite difference of stochastic_first_order_RFD
        (:373-400): (kT/delta) (N(q + delta/2 W) - N(q - delta/2 W)) W~ with
        W~ = W, translation divided by body_length, evaluated as
        A+^-1 (b - A+ A-^-1 b) on the displaced configurations."""
        import torch
        n3 = 3 * self.system.n_blobs
        f = rfd.reshape(-1, 6).clone()
        f[:, :3] /= self.body_length[:, None]
        b = torch.cat([self._zeros(n3), -f.reshape(-1)])
        A = self.aux
        xm, qm = self._move(x0, q0, rfd, -0.5 * self.rf_delta, length_scaled=True)
        sol_m = self._solve(self._at(A, xm, qm), RHS=b)
        xp, qp = self._move(x0, q0, rfd, 0.5 * self.rf_delta, length_scaled=True)
        self._at(A, xp, qp)
        drift = self._vel(self._solve(A, RHS=b - A.apply(sol_m, mode=self.mode)))
        return (self.kT / self.rf_delta) * drift

    def stochastic_first_order_RFD(self, dt):
        x0, q0 = self.x, self.q
        rfd = self.normal(6 * self.system.n_bodies)
        S = self._at(self.system, x0, q0, stochastic=True)
        noise = self._lanczos(S, math.sqrt(2.0 * self.kT / dt))
        v = self._vel(self._solve(S, noise=noise)) + self._rfd_drift(x0, q0, rfd)
        xn, qn = self._move(x0, q0, v, dt)
        return (xn, qn) if self._valid(xn, qn) else None

    def stochastic_adams_bashforth(self, dt):
        x0, q0 = self.x, self.q
        rfd = self.normal(6 * self.system.n_bodies)
        S = self._at(self.system, x0, q0, stochastic=True)
        noise = self._lanczos(S, math.sqrt(2.0 * self.kT / dt))
        v_stoch = self._vel(self._solve(S, RHS=self._zeros(S.size), noise=noise))
        v_det = self._vel(self._solve(S))
        v_stoch = v_stoch + self._rfd_drift(x0, q0, rfd)
        if self.first_step:
            v = v_det + v_stoch
        else:
            v = 1.5 * v_det - 0.5 * self.velocities_previous_step + v_stoch
        xn, qn = self._move(x0, q0, v, dt)
        if not self._valid(xn, qn):
            return None
        self.first_step = False
        self.velocities_previous_step = v_det
        return xn, qn

    def _traction(self, x0, q0, S, rfd):
        """Traction random finite difference (:650-690): [lambda; U] solves the
        mobility problem for the random force-torque -W (W = kT rfd, translation
        divided by body_length); returns (1/delta)(D M lambda - D K U) and
        -(1/delta) D K^T lambda, both from one operator apply at each
        configuration: A [lambda; U] = [M lambda - K U; -K^T lambda]."""
        import torch
        n3 = 3 * S.n_blobs
        W = rfd.reshape(-1, 6).clone()
        W[:, :3] *= self.kT / self.body_length[:, None]
        W[:, 3:] *= self.kT
        sol = self._solve(S, RHS=torch.cat([self._zeros(n3), -W.reshape(-1)]))
        xr, qr = self._move(x0, q0, rfd, self.rf_delta, length_scaled=True)
        d = self._at(self.aux, xr, qr).apply(sol, mode=self.mode) - S.apply(sol, mode=self.mode)
        d /= self.rf_delta
        return d[:n3], d[n3:]

    def stochastic_traction_EM(self, dt):
        x0, q0 = self.x, self.q
        rfd = self.normal(6 * self.system.n_bodies)
        S = self._at(self.system, x0, q0, stochastic=True)
        slip_d, force_d = self._traction(x0, q0, S, rfd)
        noise = self._lanczos(S, math.sqrt(2.0 * self.kT / dt))
        v = self._vel(self._solve(S, noise=noise + slip_d, noise_FT=force_d))
        xn, qn = self._move(x0, q0, v, dt)
        return (xn, qn) if self._valid(xn, qn) else None

    def stochastic_traction_AB(self, dt):
        import torch
        x0, q0 = self.x, self.q
        rfd = self.normal(6 * self.system.n_bodies)
        S = self._at(self.system, x0, q0, stochastic=True)
        slip_d, force_d = self._traction(x0, q0, S, rfd)
        noise = self._lanczos(S, math.sqrt(2.0 * self.kT / dt))
        v_new = self._vel(self._solve(S, noise=slip_d, noise_FT=force_d))
        v_noise = self._vel(self._solve(S, RHS=torch.cat([-noise, self._zeros(6 * S.n_bodies)])))
        if self.first_step:
            v = v_new + v_noise
        else:
            v = 1.5 * v_new + v_noise - 0.5 * self.velocities_previous_step
        xn, qn = self._move(x0, q0, v, dt)
        if not self._valid(xn, qn):
            return None
        self.first_step = False
        self.velocities_previous_step = v_new
        return xn, qn

    def _slip_scheme(self, dt, mid):
        """stochastic_Slip_Trapz (:925-1045, mid=False) and stochastic_Slip_Mid
        (:1214-1330, mid=True): the drift from a slip random finite difference
        M(q + delta W_RFD) W_slip - M W_slip with W_RFD the body velocity of the
        slip -W_slip."""
        import torch
        S0 = self.system
        n3 = 3 * S0.n_blobs
        x0, q0 = self.x, self.q
        W1 = self.normal(n3)
        W_slip = self.normal(n3)
        Wcor = W1 + self.normal(n3) if mid else None
        S = self._at(S0, x0, q0, stochastic=True)
        ws = torch.cat([W_slip, self._zeros(6 * S.n_bodies)])
        MW = S.apply(ws, mode=self.mode)  # [M W_slip; -K^T W_slip]
        noise1 = self._lanczos(S, math.sqrt((4.0 if mid else 2.0) * self.kT / dt), z=W1)
        noise_cor = self._lanczos(S, math.sqrt(self.kT / dt), z=Wcor) if mid else noise1
        v1 = self._vel(self._solve(S, noise=noise1))
        W_rfd = self._vel(self._solve(S, RHS=torch.cat([-W_slip, self._zeros(6 * S.n_bodies)])))
        xr, qr = self._move(x0, q0, W_rfd, self.rf_delta)
        d = self._at(self.aux, xr, qr).apply(ws, mode=self.mode) - MW
        d *= (1.0 if mid else 2.0) * self.kT / self.rf_delta
        rand_slip = noise_cor + d[:n3]
        xp, qp = self._move(x0, q0, v1, 0.5 * dt if mid else dt)
        if not self._valid(xp, qp):
            return None
        v2 = self._vel(self._solve(self._at(self.aux, xp, qp), noise=rand_slip, noise_FT=d[n3:]))
        v = v2 if mid else 0.5 * (v1 + v2)
        xn, qn = self._move(x0, q0, v, dt)
        return (xn, qn) if self._valid(xn, qn) else None

    def stochastic_Slip_Trapz(self, dt):
        return self._slip_scheme(dt, mid=False)

    def stochastic_Slip_Mid(self, dt):
        return self._slip_scheme(dt, mid=True)

    def close(self):
        if self._aux is not None:
            self._aux.close()
            self._aux = None
