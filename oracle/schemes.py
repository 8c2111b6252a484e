"""Oracle (test infrastructure only): numpy restatement of the reference's
GMRES-based time integrators for rigid multiblob bodies above a wall,
quaternion_integrator/quaternion_integrator_multi_bodies.py:

* deterministic_forward_euler   :75-108
* deterministic_adams_bashforth :142-185
* deterministic_midpoint        :188-259
* stochastic_EM                 :262-322
* stochastic_first_order_RFD    :326-428
* stochastic_adams_bashforth    :431-560
* stochastic_traction_EM        :626-735
* stochastic_traction_AB        :803-922
* stochastic_Slip_Trapz         :925-1045
* stochastic_Slip_Mid           :1214-1330
* solve_mobility_problem        :1441-1547 (RHS = [slip - noise; -(FT + noise_FT)],
                                  scaled to norm 1, right-preconditioned GMRES)
* check_positions               :1779-1824 (single wall: no blob below z = 0, body/body.py:118-139)

Every normal draw comes from ``normal(n)`` in the order the reference makes
them (np.random.normal, and np.random.randn inside stochastic_forcing_lanczos),
so a recorded draw sequence reproduces the reference's step.  Forces are the
default example's: gravity and wall repulsion on every blob plus blob-blob
repulsion (multi_bodies/multi_bodies_functions.py:153-189, 297-345), reduced per
body (:411-445).  Differences from the reference that change no result beyond
the solver tolerance: GMRES starts from zero (the reference warm-starts some
solves), and the preconditioner is always built at the configuration of the
solve (the reference reuses the step's first one for the corrector solves).

Pinned to tests/golden/schemes.npz.  Only tests, smoke() and bench.py's CPU
legs use it.
"""
import numpy as np

from . import forces as oforces
from . import rigid as orig


def rotation_matrix(q):
    """R(q) for a unit quaternion q = (s, p): R v = v + 2 s p x v + 2 p x (p x v)."""
    s, p = q[0], np.asarray(q[1:])
    P = np.array([[0.0, -p[2], p[1]], [p[2], 0.0, -p[0]], [-p[1], p[0], 0.0]])
    return np.eye(3) + 2.0 * s * P + 2.0 * P @ P


class Integrator:
    """One suspension of rigid bodies of blob reference coordinates r_ref
    (body b owns rows offsets[b]:offsets[b+1]), locations x (Nb,3) and
    quaternions q (Nb,4)."""

    def __init__(self, scheme, x, q, r_ref, offsets, eta, a, kT, body_length, normal, force_params,
                 tolerance=1e-8, rf_delta=1e-3, wall=True):
        self.scheme = scheme
        self.wall = wall  # False: free space, and no wall-crossing check
        self.x = np.array(x, dtype=np.float64).reshape(-1, 3)
        self.q = np.array(q, dtype=np.float64).reshape(-1, 4)
        self.r_ref = np.asarray(r_ref, dtype=np.float64).reshape(-1, 3)
        self.offsets = np.asarray(offsets, dtype=np.int64)
        self.eta, self.a, self.kT = float(eta), float(a), float(kT)
        self.body_length = np.broadcast_to(np.asarray(body_length, dtype=np.float64), (self.x.shape[0],)).copy()
        self.normal = normal
        # blob_mass, g, repulsion_strength_wall, debye_length_wall, repulsion_strength, debye_length
        self.fp = tuple(float(v) for v in force_params)
        self.tolerance = tolerance
        self.rf_delta = rf_delta
        self.Nb = self.x.shape[0]
        self.N = int(self.offsets[-1])
        self.first_step = True
        self.velocities_previous_step = None
        self.invalid_configuration_count = 0

    # -- configuration ---------------------------------------------------------
    def r_vectors(self, x, q):
        r = np.empty((self.N, 3))
        for b in range(self.Nb):
            sl = slice(self.offsets[b], self.offsets[b + 1])
            r[sl] = self.r_ref[sl] @ rotation_matrix(q[b]).T + x[b]
        return r

    def system(self, x, q):
        return orig.Rigid(self.r_vectors(x, q), x, self.offsets, self.eta, self.a, wall_present=self.wall)

    def move(self, x, q, vel, scale, length_scaled=False):
        """location + v scale (times body_length if length_scaled),
        from_rotation(w scale) * orientation."""
        v = np.asarray(vel, dtype=np.float64).reshape(-1, 6).copy()
        if length_scaled:
            v[:, :3] *= self.body_length[:, None]
        return orig.em_update(x, q, v.reshape(-1), scale)

    def valid(self, x, q):
        if not self.wall:
            return True
        ok = not bool((self.r_vectors(x, q)[:, 2] < 0.0).any())
        if not ok:
            self.invalid_configuration_count += 1
        return ok

    # -- pieces ----------------------------------------------------------------
    def force_torque(self, S):
        m, g, ew, bw, e, b = self.fp
        f = oforces.external_forces(S.r, m, self.a, g, ew, bw)
        f += oforces.blob_blob_forces(S.r, e, b, self.a)
        return oforces.body_force_torque(S.r, S.locs, self.offsets, f).reshape(-1)

    def solve(self, S, RHS=None, noise=None, noise_FT=None):
        n3 = 3 * self.N
        if RHS is None:
            FT = self.force_torque(S)
            if noise_FT is not None:
                FT = FT + noise_FT
            RHS = np.concatenate([np.zeros(n3), -FT])
        else:
            RHS = np.array(RHS, dtype=np.float64)
        if noise is not None:
            RHS[:n3] -= noise
        nrm = np.linalg.norm(RHS)
        if nrm == 0:
            return np.zeros_like(RHS)
        sol, _, _ = orig.gmres_right(S.apply, S.apply_pc, RHS / nrm, tol=self.tolerance)
        return sol * nrm

    def vel(self, sol):
        return sol[3 * self.N:]

    def lanczos(self, S, factor, z=None):
        if factor == 0.0:
            return np.zeros(3 * self.N)
        if z is None:
            z = self.normal(3 * self.N)
        w, _ = orig.lanczos(S.mobility_pc, z, factor=factor, tol=self.tolerance)
        return S.P_inv_mult(w)

    def advance_time_step(self, dt):
        while True:
            res = getattr(self, self.scheme)(dt)
            if res is not None:
                self.x, self.q = res
                return

    # -- schemes (each returns the accepted new state or None to redraw) ----------
    def deterministic_forward_euler(self, dt):
        S = self.system(self.x, self.q)
        xn, qn = self.move(self.x, self.q, self.vel(self.solve(S)), dt)
        return (xn, qn) if self.valid(xn, qn) else None

    def deterministic_adams_bashforth(self, dt):
        S = self.system(self.x, self.q)
        v = self.vel(self.solve(S))
        va = v if self.first_step else 1.5 * v - 0.5 * self.velocities_previous_step
        xn, qn = self.move(self.x, self.q, va, dt)
        if not self.valid(xn, qn):
            return None
        self.first_step = False
        self.velocities_previous_step = v
        return xn, qn

    def deterministic_midpoint(self, dt):
        x0, q0 = self.x, self.q
        v = self.vel(self.solve(self.system(x0, q0)))
        xm, qm = self.move(x0, q0, v, 0.5 * dt)
        if not self.valid(xm, qm):
            return None
        vm = self.vel(self.solve(self.system(xm, qm)))
        xn, qn = self.move(x0, q0, vm, dt)
        return (xn, qn) if self.valid(xn, qn) else None

    def stochastic_EM(self, dt):
        S = self.system(self.x, self.q)
        noise = self.lanczos(S, np.sqrt(2.0 * self.kT / dt))
        xn, qn = self.move(self.x, self.q, self.vel(self.solve(S, noise=noise)), dt)
        return (xn, qn) if self.valid(xn, qn) else None

    def _rfd_drift(self, x0, q0, rfd):
        """(kT / delta) (N(q + delta/2 W) - N(q - delta/2 W)) W~, the two-solve RFD
        of stochastic_first_order_RFD: W~ = W with the translation divided by
        body_length, displacements scaled by body_length."""
        n3 = 3 * self.N
        force_rfd = rfd.reshape(-1, 6).copy()
        force_rfd[:, :3] /= self.body_length[:, None]
        force_rfd = force_rfd.reshape(-1)
        b = np.concatenate([np.zeros(n3), -force_rfd])
        xm, qm = self.move(x0, q0, rfd, -0.5 * self.rf_delta, length_scaled=True)
        sol_m = self.solve(self.system(xm, qm), RHS=b)
        xp, qp = self.move(x0, q0, rfd, 0.5 * self.rf_delta, length_scaled=True)
        Sp = self.system(xp, qp)
        drift = self.vel(self.solve(Sp, RHS=b - Sp.apply(sol_m)))
        return (self.kT / self.rf_delta) * drift

    def stochastic_first_order_RFD(self, dt):
        x0, q0 = self.x, self.q
        rfd = self.normal(6 * self.Nb)
        S = self.system(x0, q0)
        noise = self.lanczos(S, np.sqrt(2.0 * self.kT / dt))
        v = self.vel(self.solve(S, noise=noise)) + self._rfd_drift(x0, q0, rfd)
        xn, qn = self.move(x0, q0, v, dt)
        return (xn, qn) if self.valid(xn, qn) else None

    def stochastic_adams_bashforth(self, dt):
        x0, q0 = self.x, self.q
        rfd = self.normal(6 * self.Nb)
        S = self.system(x0, q0)
        noise = self.lanczos(S, np.sqrt(2.0 * self.kT / dt))
        v_stoch = self.vel(self.solve(S, RHS=np.zeros(S.size), noise=noise))
        v_det = self.vel(self.solve(S))
        v_stoch = v_stoch + self._rfd_drift(x0, q0, rfd)
        if self.first_step:
            v = v_det + v_stoch
        else:
            v = 1.5 * v_det - 0.5 * self.velocities_previous_step + v_stoch
        xn, qn = self.move(x0, q0, v, dt)
        if not self.valid(xn, qn):
            return None
        self.first_step = False
        self.velocities_previous_step = v_det
        return xn, qn

    def _traction(self, x0, q0, S, rfd):
        """Traction RFD pieces (rand_slip without the Brownian slip, rand_force):
        (1/delta) (D_x M lambda - D_x K U) and -(1/delta) D_x K^T lambda, with
        [lambda; U] the solution for the random force-torque -W."""
        n3 = 3 * self.N
        W = rfd.reshape(-1, 6).copy()
        W[:, :3] *= self.kT / self.body_length[:, None]
        W[:, 3:] *= self.kT
        sol = self.solve(S, RHS=np.concatenate([np.zeros(n3), -W.reshape(-1)]))
        xr, qr = self.move(x0, q0, rfd, self.rf_delta, length_scaled=True)
        Sr = self.system(xr, qr)
        d = Sr.apply(sol) - S.apply(sol)  # [D_x M lambda - D_x K U; -D_x K^T lambda]
        return d[:n3] / self.rf_delta, d[n3:] / self.rf_delta

    def stochastic_traction_EM(self, dt):
        x0, q0 = self.x, self.q
        rfd = self.normal(6 * self.Nb)
        S = self.system(x0, q0)
        slip_d, force_d = self._traction(x0, q0, S, rfd)
        noise = self.lanczos(S, np.sqrt(2.0 * self.kT / dt))
        v = self.vel(self.solve(S, noise=noise + slip_d, noise_FT=force_d))
        xn, qn = self.move(x0, q0, v, dt)
        return (xn, qn) if self.valid(xn, qn) else None

    def stochastic_traction_AB(self, dt):
        x0, q0 = self.x, self.q
        rfd = self.normal(6 * self.Nb)
        S = self.system(x0, q0)
        slip_d, force_d = self._traction(x0, q0, S, rfd)
        noise = self.lanczos(S, np.sqrt(2.0 * self.kT / dt))
        v_new = self.vel(self.solve(S, noise=slip_d, noise_FT=force_d))
        v_noise = self.vel(self.solve(S, RHS=np.concatenate([-noise, np.zeros(6 * self.Nb)])))
        if self.first_step:
            v = v_new + v_noise
        else:
            v = 1.5 * v_new + v_noise - 0.5 * self.velocities_previous_step
        xn, qn = self.move(x0, q0, v, dt)
        if not self.valid(xn, qn):
            return None
        self.first_step = False
        self.velocities_previous_step = v_new
        return xn, qn

    def _slip(self, dt, mid):
        """stochastic_Slip_Trapz (mid=False) and stochastic_Slip_Mid (mid=True)."""
        n3 = 3 * self.N
        x0, q0 = self.x, self.q
        W1 = self.normal(n3)
        W_slip = self.normal(n3)
        Wcor = W1 + self.normal(n3) if mid else None
        S = self.system(x0, q0)
        MW = S.apply(np.concatenate([W_slip, np.zeros(6 * self.Nb)]))  # [M W; -K^T W]
        noise1 = self.lanczos(S, np.sqrt((4.0 if mid else 2.0) * self.kT / dt), z=W1)
        noise_cor = self.lanczos(S, np.sqrt(self.kT / dt), z=Wcor) if mid else noise1
        v1 = self.vel(self.solve(S, noise=noise1))
        W_rfd = self.vel(self.solve(S, RHS=np.concatenate([-W_slip, np.zeros(6 * self.Nb)])))
        xr, qr = self.move(x0, q0, W_rfd, self.rf_delta)
        MW_r = self.system(xr, qr).apply(np.concatenate([W_slip, np.zeros(6 * self.Nb)]))
        c = (1.0 if mid else 2.0) * self.kT / self.rf_delta
        rand_slip = noise_cor + c * (MW_r[:n3] - MW[:n3])
        rand_force = c * (MW_r[n3:] - MW[n3:])  # -c (K_r^T W - K^T W)
        xp, qp = self.move(x0, q0, v1, 0.5 * dt if mid else dt)
        if not self.valid(xp, qp):
            return None
        v2 = self.vel(self.solve(self.system(xp, qp), noise=rand_slip, noise_FT=rand_force))
        v = v2 if mid else 0.5 * (v1 + v2)
        xn, qn = self.move(x0, q0, v, dt)
        return (xn, qn) if self.valid(xn, qn) else None

    def stochastic_Slip_Trapz(self, dt):
        return self._slip(dt, mid=False)

    def stochastic_Slip_Mid(self, dt):
        return self._slip(dt, mid=True)
