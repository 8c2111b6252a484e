"""Blob and body forces on the GPU: the right-hand side of the mobility problem.

Drop-ins for the reference's force functions (multi_bodies/forces_pycuda.py,
multi_bodies/multi_bodies_functions.py), same names, keyword arguments and
return shapes:

* calc_blob_blob_forces_pycuda(r_vectors, periodic_length=, repulsion_strength=,
  debye_length=, blob_radius=) -> (N, 3) soft blob-blob repulsion
  (also under the numba and python implementation names), and
  calc_blob_blob_forces_tree_numba (pairs within 2a + 30 b);
* blob_external_forces(r_vectors, blob_mass=, blob_radius=, g=,
  repulsion_strength_wall=, debye_length_wall=) -> (N, 3) gravity and wall repulsion;
* force_torque_calculator_sort_by_bodies(system, r_vectors, ...) -> (2 Nb, 3)
  [F_1, T_1, F_2, T_2, ...]: blob forces summed per body and their moments
  about the body locations, through the rigid handle's K^T.

numpy in -> numpy out; CUDA torch tensors stay on the device.
"""
import numpy as np

from . import _native


def _device_of(*xs):
    import torch
    for x in xs:
        if isinstance(x, torch.Tensor) and x.is_cuda:
            return x.device, True
    for x in xs:
        if isinstance(x, torch.Tensor):
            raise ValueError("torch inputs must be CUDA tensors")
    return torch.device("cuda", torch.cuda.current_device()), False


def _blob_blob(r, f, L, eps, b, a, accumulate, dev, cutoff=0.0):
    import torch
    Lh = np.ascontiguousarray(np.zeros(3) if L is None else np.asarray(L, dtype=np.float64).reshape(3))
    with torch.cuda.device(dev):
        _native.call("rmw_blob_blob_forces", r.data_ptr(), f.data_ptr(), r.shape[0], float(eps), float(b), float(a),
                     float(cutoff), Lh.ctypes.data, 1 if accumulate else 0,
                     torch.cuda.current_stream(dev).cuda_stream)


def _external(r, f, m, a, g, e, b, accumulate, dev):
    import torch
    with torch.cuda.device(dev):
        _native.call("rmw_blob_external_forces", r.data_ptr(), f.data_ptr(), r.shape[0], float(m), float(a), float(g),
                     float(e), float(b), 1 if accumulate else 0, torch.cuda.current_stream(dev).cuda_stream)


def calc_blob_blob_forces_pycuda(r_vectors, *args, **kwargs):
    """Blob-blob repulsion, shape (N, 3) (multi_bodies/forces_pycuda.py:148-180)."""
    import torch
    dev, on_device = _device_of(r_vectors)
    r = torch.as_tensor(r_vectors, dtype=torch.float64, device=dev).reshape(-1, 3).contiguous()
    f = torch.empty_like(r)
    _blob_blob(r, f, kwargs.get("periodic_length"), kwargs.get("repulsion_strength"), kwargs.get("debye_length"),
               kwargs.get("blob_radius"), False, dev)
    return f if on_device else f.cpu().numpy()


calc_blob_blob_forces_numba = calc_blob_blob_forces_pycuda
calc_blob_blob_forces_python = calc_blob_blob_forces_pycuda


def calc_blob_blob_forces_tree_numba(r_vectors, *args, **kwargs):
    """Blob-blob repulsion over the pairs within d_max = 2a + 30 b, the
    truncation of the reference's neighbour-list version
    (multi_bodies/forces_numba.py:228-270); no neighbour list is needed on the
    GPU: the all-pairs kernel screens by distance."""
    import torch
    dev, on_device = _device_of(r_vectors)
    r = torch.as_tensor(r_vectors, dtype=torch.float64, device=dev).reshape(-1, 3).contiguous()
    f = torch.empty_like(r)
    a, b = kwargs.get("blob_radius"), kwargs.get("debye_length")
    _blob_blob(r, f, kwargs.get("periodic_length"), kwargs.get("repulsion_strength"), b, a, False, dev,
               cutoff=2 * a + 30 * b)
    return f if on_device else f.cpu().numpy()


def blob_external_forces(r_vectors, *args, **kwargs):
    """Gravity and wall repulsion, shape (N, 3) (multi_bodies_functions.py:153-189)."""
    import torch
    dev, on_device = _device_of(r_vectors)
    r = torch.as_tensor(r_vectors, dtype=torch.float64, device=dev).reshape(-1, 3).contiguous()
    f = torch.empty_like(r)
    _external(r, f, kwargs.get("blob_mass"), kwargs.get("blob_radius"), kwargs.get("g"),
              kwargs.get("repulsion_strength_wall"), kwargs.get("debye_length_wall"), False, dev)
    return f if on_device else f.cpu().numpy()


def force_torque_calculator_sort_by_bodies(system, r_vectors, *args, **kwargs):
    """[F_1, T_1, F_2, T_2, ...] of shape (2 Nb, 3) for the bodies of `system`
    (rigid.RigidSystem, configuration already set): external plus blob-blob
    blob forces (the default example's calc_one_blob_forces and
    calc_blob_blob_forces), reduced per body with K^T
    (multi_bodies_functions.py:411-445).  Keyword arguments as the reference's
    (blob_mass defaults to 1, blob_radius to the system's a); without
    debye_length the blob-blob forces are left out."""
    import torch
    dev = system.device
    on_device = isinstance(r_vectors, torch.Tensor)
    r = torch.as_tensor(r_vectors, dtype=torch.float64, device=dev).reshape(-1, 3).contiguous()
    a = kwargs.get("blob_radius", system.a)
    f = torch.empty_like(r)
    _external(r, f, kwargs.get("blob_mass", 1.0), a, kwargs.get("g", 0.0), kwargs.get("repulsion_strength_wall", 0.0),
              kwargs.get("debye_length_wall", 1.0), False, dev)
    if kwargs.get("debye_length") is not None:
        _blob_blob(r, f, kwargs.get("periodic_length"), kwargs.get("repulsion_strength", 0.0),
                   kwargs.get("debye_length"), a, True, dev)
    ft = system.KT_mult(f.reshape(-1)).reshape(-1, 3)
    return ft if on_device else ft.cpu().numpy()
