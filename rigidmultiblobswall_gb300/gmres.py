"""Name-compatible home of the reference's quaternion_integrator/gmres.py
(gmres :166-195, right_gmres :197-230), which returns (x, info, resnorms).

The reference wraps scipy's private Fortran GMRES; here both names run the
device GMRES of krylov.gmres with the semantics of
general_application_utils.gmres: convergence='resid' stops on the true
residual |b - A x| <= tol |b| (right preconditioner M = P^-1 when given),
convergence='presid' on the preconditioned residual |M (b - A x)| <= tol |M b|
(left preconditioner).  resnorms holds the relative residual estimate of
every iteration; verbose prints them as the reference's counter does.
"""
from . import krylov

_KEYS = ("x0", "tol", "restart", "maxiter", "M")


def _solve(A, b, verbose, side, kwargs):
    unknown = set(kwargs) - set(_KEYS) - {"callback", "restrt", "xtype", "atol"}
    if unknown:
        raise TypeError("unexpected keyword arguments: %s" % ", ".join(sorted(unknown)))
    resnorms = []
    user_cb = kwargs.get("callback")

    def cb(rk):
        resnorms.append(rk)
        if verbose:
            print("iter %3i\trk = %s" % (len(resnorms), str(rk)))
        if user_cb is not None:
            user_cb(rk)

    x, info = krylov.gmres(A, b, x0=kwargs.get("x0"), tol=kwargs.get("tol", 1e-05), restart=kwargs.get("restart"),
                           maxiter=kwargs.get("maxiter"), M=kwargs.get("M"), callback=cb,
                           restrt=kwargs.get("restrt"), PC_side=side)
    return x, info, resnorms


def gmres(A, b, verbose=False, convergence="resid", **kwargs):
    if convergence not in ("resid", "presid"):
        raise Exception("convergence must be set to 'resid' or 'presid'")
    side = "left" if (convergence == "presid" and kwargs.get("M") is not None) else "right"
    return _solve(A, b, verbose, side, kwargs)


def right_gmres(A, b, verbose=False, **kwargs):
    if "M" not in kwargs:
        raise Exception("M must be a kwarg for right_gmres")
    return _solve(A, b, verbose, "right", kwargs)
