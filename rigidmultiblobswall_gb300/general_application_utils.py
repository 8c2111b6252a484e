"""Name-compatible home of the reference's general_application_utils.gmres
(general_application_utils.py:514-635); the solver is rigidmultiblobswall_gb300.krylov.gmres."""
from .krylov import gmres  # noqa: F401
