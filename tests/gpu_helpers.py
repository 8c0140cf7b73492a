"""Shared helpers of the GPU parity tests."""
import numpy as np

import oracle.asm_oracle as O


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def oracle_params(kw, extras=None):
    p = O.OracleParams(**kw)
    for k, v in (extras or {}).items():
        setattr(p, k, v)
    return p


def solver_params(kw, extras=None):
    from angularspectrum_heterogeneous_gb300 import SolverParams
    p = SolverParams(**kw)
    for k, v in (extras or {}).items():
        setattr(p, k, v)
    return p


# Tolerances of the parity tests (relative L2 against the FP64 oracle):
# the spec bar is 1e-4 on the field and 1e-3 on pnp/ppp/pI.  pIloss is a
# difference of two nearly equal sums (I_before - I_after) and carries the
# FP32 rounding of both; it gets 1e-2.
TOL = {"field": 1e-4, "pnp": 1e-3, "ppp": 1e-3, "pI": 1e-3, "pIloss": 1e-2, "pax": 1e-3}
KEYS = ["field", "pnp", "ppp", "pI", "pIloss", "zaxis", "pax"]
