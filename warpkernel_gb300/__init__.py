"""GB300-native WPK1/WPK2 sparse matrix-vector multiply (sm_103a).

The product is libwarpkernel_gb300.so (C ABI in include/wk_capi.h); this
package is a thin Python binding over it that mirrors the reference's
warpkernel.hpp classes.
"""
from .wpk import (WK_ORDER_EXACT, WK_ORDER_FAST, engine, profiler, stats, structure,  # noqa: F401
                  structure2)
from ._lib import WKError, load  # noqa: F401
from . import fe  # noqa: F401
