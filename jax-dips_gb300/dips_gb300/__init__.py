"""dips_gb300: the JAX-DIPS NBM jump-condition FV residual hot path on GB300 (sm_103a).

Host-side mirror of the reference's interface for this path:
``solvers.poisson.trainer.setup -> init_fn -> solve_fn`` (``dips_gb300.trainer``) and
``nn.configure.get_model`` (``dips_gb300.nn``); the compute runs in the CUDA library
declared in include/dips.h.
"""

__version__ = "0.1.0"


def build(force=False, verbose=False):
    from . import _lib

    return _lib.build(force=force, verbose=verbose)
