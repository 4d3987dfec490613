"""GB300-native (sm_103a) phase-space upwind-DG advection path with the
interface of hyper.deal's AdvectionOperation / LowStorageRungeKuttaIntegrator.

The compute path is the CUDA library built from ``csrc/`` and reached through
the C ABI in ``include/hyperdeal_gb300.h``; this package is its Python host
side (used by the tests and the benchmark).
"""
from ._lib import HdError, load as load_library, lib_path  # noqa: F401
from .build import build as build_library  # noqa: F401

__version__ = "0.1.0"


def __getattr__(name):
    # the torch-based host API is imported lazily so that building and the
    # symbol checks do not need torch
    if name in ("AdvectionOperation", "AdvectionParameters", "Function", "LowStorageRungeKuttaIntegrator",
                "TimeLoop", "VectorTools", "compute_critical_time_step", "time_step_rule", "advection"):
        import importlib
        mod = importlib.import_module(__name__ + ".advection")
        return mod if name == "advection" else getattr(mod, name)
    if name in ("VlasovPoissonParameters", "VlasovPoissonOperation", "perturbed_maxwellian", "vlasov_poisson"):
        import importlib
        mod = importlib.import_module(__name__ + ".vlasov_poisson")
        return mod if name == "vlasov_poisson" else getattr(mod, name)
    raise AttributeError(name)
