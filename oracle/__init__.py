"""CPU oracle for the muxi_spmv hot path -- TEST INFRASTRUCTURE.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
package, always as the checker or as the timed CPU reference path.  The
library (muxi_spmv_gb300) never imports it.
"""
from .oracle import *  # noqa: F401,F403
