"""CPU oracle of Spike's clock-driven step (TEST INFRASTRUCTURE ONLY).

Imported only by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
leg, as the checker of the CUDA engine; the engine never calls it.
"""
from .binding import OracleNet, oracle_lib  # noqa: F401
