"""GB300-native per-iteration structured-grid solver step (aither path)."""
from ._lib import Batch, Context, Server, Setup, AthError, PREC_FP64, PREC_MIXED  # noqa: F401
