"""gspan_gb300: GPU frequent-subgraph mining (gSpan, MNI support) for one GB300.

Typical use mirrors the reference's ``fsm(graph, k, min_support)``
(gspan.h:41 of haozixu/gSpan)::

    from gspan_gb300 import Miner, load_bin, format_pattern
    g = load_bin("graph.bin")
    with Miner() as m:
        patterns, stats = m.fsm(g, k=3, min_support=300)
    for code, sup in patterns:
        print(format_pattern(code, sup))

The graph generators and file readers (``datagen``) are plain numpy and load
no native code.  Every other name (``Miner``, ``Server``, ``is_canonical`` ...)
lives in ``capi``, the ctypes view of ``_lib/libgspan_gb300.so``; the library is
loaded the first time one of them is used, and that use fails loudly with
ImportError if the library has not been built.  There is no CPU fallback.
"""
from __future__ import annotations

import importlib

from . import datagen  # noqa: F401
from .datagen import CSR, load_bin  # noqa: F401  (re-exported)


def __getattr__(name: str):
    # PEP 562: names of the C ABI view resolve on first use.
    if name.startswith("__"):
        raise AttributeError(name)
    capi = importlib.import_module(__name__ + ".capi")
    try:
        return getattr(capi, name)
    except AttributeError:
        raise AttributeError(f"module 'gspan_gb300' has no attribute {name!r}") from None
