"""GB300-native WPK1/WPK2 sparse matrix-vector multiply (sm_103a).

The product is libwarpkernel_gb300.so (C ABI in include/wk_capi.h); this
package is a thin Python binding over it that mirrors the reference's
warpkernel.hpp classes.
"""
from .wpk import (WK_ORDER_EXACT, WK_ORDER_FAST, csr_matrix, engine, profiler,  # noqa: F401
                  read_matrix_market_file, stats, structure, structure2)
from ._lib import WK_ABL_NOCOALESCE, WK_ABL_NOSORT, WKError, load  # noqa: F401
from . import fe  # noqa: F401
