"""GB300-native (sm_103a) hot path of the quasi-dynamic antiplane earthquake
cycle of QDEqCycle_FDM: multigrid displacement solve, fault stress, Newton
for slip rate, aging law and the adaptive RK43 stage pipeline, behind the C
ABI declared in ``include/qdeq.h``.
"""
from . import config, problem  # noqa: F401

__all__ = ["config", "problem", "api", "build"]
