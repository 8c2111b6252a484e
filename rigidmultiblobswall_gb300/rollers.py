"""Rollers (single blobs driven at a prescribed angular velocity) on the GPU,
following quaternion_integrator/quaternion_integrator_rollers.py:

* compute_deterministic_velocity_and_torque (:905-983): with prescribed
  kinematics the torques solve M_WT T = omega - M_WF F by GMRES (no
  preconditioner, RHS-relative tolerance) and the velocities are
  U = M_UF F + M_UT T, all in rmw_rollers_velocity_and_torque; with free
  kinematics the torques are omega 8 pi eta a^3 (get_torque, :1586-1597);
* QuaternionIntegratorRollers.deterministic_forward_euler (:119-152): x += U dt,
  a step that puts a roller below z = 0 is rejected and recomputed (the
  reference recomputes it unchanged as well), rollers below z = a are
  counted in wall_overlaps.

Forces are device (N, 3) arrays from calc_one_blob_forces / calc_blob_blob_forces
callables (e.g. forces.blob_external_forces and
forces.calc_blob_blob_forces_pycuda with keyword arguments bound), as the
reference's integrator holds them.
"""
import ctypes
import math

import numpy as np

from . import _native

_MODES = {"fp64": _native.MODE_FP64, "mixed": _native.MODE_MIXED, "df64": _native.MODE_DF64}


def compute_deterministic_velocity_and_torque(r_vectors, force, omega, eta, a, periodic_length=None, tolerance=1e-8,
                                              domain="single_wall", free_kinematics=False, restart=20,
                                              maxiter=1000, mode="fp64"):
    """(velocity (3N,), torque (3N,), GMRES iterations) of N rollers at r_vectors
    under blob forces `force`, every roller turning at `omega` (a 3-vector or one
    per roller).  CUDA tensors stay on the device; numpy in -> numpy out."""
    import torch
    if domain not in ("single_wall", "no_wall"):
        raise NotImplementedError("rollers are available above a single wall or in free space")
    is_t = any(type(x).__module__.startswith("torch") for x in (r_vectors, force, omega))
    dev = torch.device("cuda", torch.cuda.current_device())
    for x in (r_vectors, force, omega):
        if type(x).__module__.startswith("torch") and x.is_cuda:
            dev = x.device
    r = torch.as_tensor(r_vectors, dtype=torch.float64, device=dev).reshape(-1, 3).contiguous()
    n = r.shape[0]
    f = torch.as_tensor(force, dtype=torch.float64, device=dev).reshape(-1).contiguous()
    w = torch.as_tensor(omega, dtype=torch.float64, device=dev).reshape(-1, 3).expand(n, 3).reshape(-1).contiguous()
    if f.numel() != 3 * n:
        raise ValueError("force must have 3N entries")
    L = np.zeros(3) if periodic_length is None else np.ascontiguousarray(periodic_length, dtype=np.float64)
    vel = torch.empty(3 * n, dtype=torch.float64, device=dev)
    its = 0
    with torch.cuda.device(dev):
        stream = torch.cuda.current_stream(dev).cuda_stream
        if free_kinematics:
            from . import mobility as mb
            tq = w * (8.0 * math.pi * eta * a ** 3)
            kw = {"periodic_length": L, "mode": mode}
            if domain == "single_wall":
                vel = mb.wall_force_torque(r, f, tq, eta, a, with_rotation=False, **kw)
            else:
                vel = mb.no_wall_product("uf", r, f, eta, a, **kw) + mb.no_wall_product("ut", r, tq, eta, a, **kw)
        else:
            tq = torch.empty(3 * n, dtype=torch.float64, device=dev)
            it = ctypes.c_int(0)
            rr = ctypes.c_double(0.0)
            rc = _native.load().rmw_rollers_velocity_and_torque(
                r.data_ptr(), f.data_ptr(), w.data_ptr(), vel.data_ptr(), tq.data_ptr(), n, float(eta), float(a),
                L.ctypes.data_as(ctypes.c_void_p), 1 if domain == "single_wall" else 0, float(tolerance),
                int(restart), int(maxiter), _MODES[mode], stream, ctypes.byref(it), ctypes.byref(rr))
            if rc != _native.RMW_ERR_NOT_CONVERGED:
                _native.check(rc)
            its = it.value
    if is_t:
        return vel, tq, its
    return vel.cpu().numpy(), tq.cpu().numpy(), its


class QuaternionIntegratorRollers:
    """Deterministic rollers on the device: state `x` (N, 3) roller positions.
    Attributes as the reference's integrator: eta, a, omega_one_roller,
    free_kinematics ('True' / 'False'), domain, periodic_length, tolerance,
    hydro_interactions (1: full hydrodynamics), calc_one_blob_forces and
    calc_blob_blob_forces (callables r (N,3) -> (N,3)), and the counters
    det_iterations_count, invalid_configuration_count, wall_overlaps."""

    def __init__(self, x, scheme="deterministic_forward_euler", tolerance=1e-8, domain="single_wall", mode="fp64"):
        import torch
        self.x = torch.as_tensor(x, dtype=torch.float64, device="cuda").reshape(-1, 3).clone()
        self.scheme = scheme
        self.tolerance = tolerance
        self.domain = domain
        self.mode = mode
        self.eta = None
        self.a = None
        self.omega_one_roller = np.zeros(3)
        self.free_kinematics = "True"
        self.hydro_interactions = 1
        self.periodic_length = None
        self.calc_one_blob_forces = None
        self.calc_blob_blob_forces = None
        self.det_iterations_count = 0
        self.invalid_configuration_count = 0
        self.wall_overlaps = 0

    def advance_time_step(self, dt, *args, **kwargs):
        return getattr(self, self.scheme.replace("_rollers", ""))(dt, *args, **kwargs)

    def _forces(self):
        import torch
        f = torch.zeros_like(self.x)
        for fn in (self.calc_one_blob_forces, self.calc_blob_blob_forces):
            if fn is not None:
                f = f + torch.as_tensor(fn(self.x), dtype=torch.float64, device=self.x.device).reshape(-1, 3)
        return f

    def compute_deterministic_velocity_and_torque(self):
        if self.hydro_interactions != 1:
            raise NotImplementedError("only rollers with hydrodynamic interactions are on this path")
        u, t, its = compute_deterministic_velocity_and_torque(
            self.x, self._forces(), self.omega_one_roller, self.eta, self.a, periodic_length=self.periodic_length,
            tolerance=self.tolerance, domain=self.domain, free_kinematics=(self.free_kinematics != "False"),
            mode=self.mode)
        self.det_iterations_count += its
        return u, t

    def deterministic_forward_euler(self, dt, *args, max_retries=10, **kwargs):
        for _ in range(max_retries):
            u, _ = self.compute_deterministic_velocity_and_torque()
            xn = self.x + dt * u.reshape(-1, 3)
            if self.domain != "single_wall" or not bool((xn[:, 2] < 0.0).any()):
                self.x = xn
                if self.domain == "single_wall":
                    self.wall_overlaps += int((xn[:, 2] < self.a).sum())
                return
            self.invalid_configuration_count += 1
        raise RuntimeError("rollers step rejected %d times in a row" % max_retries)
