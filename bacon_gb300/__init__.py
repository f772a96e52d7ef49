"""bacon_gb300 — a GB300-native (sm_103a) batched initial-value-problem engine
with the builder/solver API of the Rust crate bacon-sci (aftix/bacon).

``bacon_gb300.ivp`` holds the builder mirror (RungeKutta45, RungeKutta23),
``bacon_gb300.engine`` the low-level batched calls over the C ABI of
``include/bacon_gb300.h``; the native library is built by
``bacon_gb300.build_ext``.
"""
__version__ = "0.1.0"


def library_path() -> str:
    from ._capi import LIB_PATH
    return LIB_PATH
