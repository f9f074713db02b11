"""Operator namespace mirroring brainpy.math.{event,sparse,jitconn}."""
from . import event  # noqa: F401
