"""Name-compatible home of the reference's stochastic_forcing.stochastic_forcing_lanczos
(stochastic_forcing/stochastic_forcing.py:112-264); the solver is
rigidmultiblobswall_gb300.krylov.stochastic_forcing_lanczos."""
from .krylov import stochastic_forcing_lanczos  # noqa: F401
