"""GB300-native per-iteration structured-grid solver step (aither path)."""
from ._lib import (BATCH_FAST_FACES, BATCH_MATRIX_RESID, PREC_FP64, PREC_MIXED,  # noqa: F401
                   AthError, Batch, Context, Server, Setup)
