"""ctwin_gb300: GB300-native engine for galloty/ctwin's PRP squaring engine and
modular-root sieve, behind a C ABI (include/ctwin_gb300.h)."""
from ._native import CtwError, lib
from .pool import Batch, Pool, Server, autotune, two_primes
from .prp import PrpEngine, prp_test
from .sieve import Sieve, sieve_pass

__all__ = ["CtwError", "lib", "PrpEngine", "prp_test", "Pool", "Batch", "Server", "autotune", "two_primes", "Sieve", "sieve_pass"]
