"""GB300-native per-iteration structured-grid solver step (aither path)."""
from ._lib import (BATCH_FAST_FACES, BATCH_MATRIX_RESID, BATCH_OUTPUT_GRADS,  # noqa: F401
                   PREC_FP64, PREC_MIXED, AthError, Batch, Context, Server, Setup)
