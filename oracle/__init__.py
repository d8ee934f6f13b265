"""FP64 CPU oracle of the contact-surface path — test infrastructure only.

Only tests/, __graft_entry__.smoke() and bench.py's CPU legs import this
package, as the checker.  Parity status: unpinned (see oracle.h).
"""
from .oracle import Oracle, build, curved_select, curved_update, generate_mesh, load, taxel_sensor

__all__ = ["Oracle", "build", "curved_select", "curved_update", "generate_mesh", "load", "taxel_sensor"]
