"""minibwa_gb300: GB300-native ksw2 extension / local alignment (minibwa's DP hot path).

The product is libksw2gpu.so (CUDA for sm_103a behind a C ABI, see include/ksw2.h and
include/ksw2_gb300.h).  This package is its Python host layer: ctypes bindings, numpy
job/result layouts, and the synthetic workloads of the benchmark configurations.
There is no CPU code path: loading fails loudly when the library is missing.
"""
from .lib import (  # noqa: F401
    EXT_JOB,
    EXT_RESULT,
    LL_JOB,
    LL_RESULT,
    RESCUE_JOB,
    RESCUE_OPT,
    RESCUE_RESULT,
    KSW_EZ_APPROX_DROP,
    KSW_EZ_APPROX_MAX,
    KSW_EZ_EXTZ_ONLY,
    KSW_EZ_GENERIC_SC,
    KSW_EZ_REV_CIGAR,
    KSW_EZ_RIGHT,
    KSW_EZ_SCORE_ONLY,
    KSW_LL_STOP,
    KSW_LL_SUBO,
    Context,
    Graph,
    Reference,
    Server,
    ExtBatch,
    LLBatch,
    KswExtz,
    KswLLRst,
    gen_nt4_mat,
    lib_path,
    load_library,
    ksw_extz2_sse,
    ksw_extd2_sse,
    ksw_ll_qinit,
    ksw_ll_u8_core,
    ksw_ll_i16_core,
    ksw_ll_i16,
)
