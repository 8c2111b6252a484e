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
    rhs = torch.zeros(sys_.size, dtype=torch.float64, device=sys_.device)
    if slip is not None:
        rhs[:n3] = torch.as_tensor(slip, dtype=torch.float64, device=sys_.device).reshape(-1)
    if noise is not None:
        rhs[:n3] -= torch.as_tensor(noise, dtype=torch.float64, device=sys_.device).reshape(-1)
    rhs[n3:] = -torch.as_tensor(force_torque, dtype=torch.float64, device=sys_.device).reshape(-1)
    return rhs


def solve_mobility_problem(sys_, force_torque, slip=None, noise=None, tol=1e-8, restart=60, maxiter=1000,
                           mode="fp64"):
    """Solution [lambda; U] of the mobility problem.  The RHS is scaled to norm 1
    before GMRES and the solution scaled back, as the reference does.
    Returns (solution, info, iterations, relative residual)."""
    rhs = mobility_rhs(sys_, force_torque, slip, noise)
    nrm = float(rhs.norm())
    if nrm == 0.0:
        return rhs.clone(), 0, 0, 0.0
    sol, info, its, rr = sys_.solve(rhs / nrm, tol=tol, restart=restart, maxiter=maxiter, mode=mode)
    return sol * nrm, info, its, rr


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
            s.build_pc(stochastic=True)
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
