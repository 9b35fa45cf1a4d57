"""rebop_gb300: GB300-native ensemble engine for rebop's run-time Gillespie path.

Drop-in surfaces:
  * ``rebop_gb300.Gillespie``             -- Python ``rebop.Gillespie``
  * ``rebop_gb300.api.Gillespie``/``Rate`` -- Rust ``rebop::gillespie`` API
  * ``rebop_gb300.define_system``         -- Rust ``define_system!`` macro
the batched entry points ``Gillespie.run_ensemble`` /
``api.Network.run_ensemble``, and ``api.Batch`` for many networks and
parameter sets in one CUDA graph.  All compute runs in hand-written sm_103a CUDA
behind the C ABI of include/rebop_gb300.h; there is no CPU fallback.
"""

from . import api
from ._lib import EngineError, lib as _lib
from .api import Batch, Network, Rate
from .gillespie import Gillespie
from .macro import define_system

__version__: str = _lib.rb_version().decode()

__all__ = ("Batch", "Gillespie", "Network", "Rate", "api", "define_system", "EngineError", "__version__")
