"""GB300-native exact big-integer multiplication: products, squares and dense
convolutions of 64-bit limb vectors through multi-prime NTTs in hand-written
sm_103a CUDA, behind the call shapes of ntt_anafis's MulPlan/MulWorkspace and
ConvPlan/ConvWorkspace."""
from .api import (  # noqa: F401
    ConvPlan,
    GpuConvWorkspace,
    GpuBatch,
    GpuMulWorkspace,
    Request,
    MulPlan,
    get_split,
    set_basecase_limit,
    load_splits,
    save_splits,
    set_split,
    split_range,
    tune_splits,
    exported_symbols,
    kernel_launches,
    last_error,
    lookback_timeouts,
    debug_stall_lookback,
    STATUS_BOUND,
    STATUS_LOOKBACK,
    library,
)
from .field import CrtPair, PrimeField  # noqa: F401
from .operands import operand  # noqa: F401

__version__ = "0.1.0"
