"""Operator namespace mirroring brainpy.math.{event,sparse,jitconn}."""
from . import event  # noqa: F401
from . import jitconn  # noqa: F401
from . import sparse  # noqa: F401
