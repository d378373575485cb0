"""sarlabtdc -- GB300-native time-domain correlation SAR processor.

Re-exports the ``_sarlabtdc`` module (py-sarlabtdc/sarlabtdc/__init__.py:31 does
``from _sarlabtdc import *``). The reference's Windows DLL-directory shim
(``__init__.py:9-29``) has no counterpart: the engine is one in-tree shared
library loaded by path.
"""
from _sarlabtdc import *  # noqa: F401,F403
from _sarlabtdc import TdcProcessor  # noqa: F401

__all__ = ["TdcProcessor"]
