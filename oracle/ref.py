"""Loader for the reference adrt package, compiled from its own sources.

TEST INFRASTRUCTURE ONLY.  ``make -C oracle ref`` compiles the reference's
CPython extension from the reference checkout into ``oracle/_ref/``; this
module imports the reference's Python package from that checkout with the
compiled extension attached.  It is available only on a machine that has the
reference checkout (not on the GPU host); callers must handle ``None``.
"""

from __future__ import annotations

import glob
import importlib.machinery
import importlib.util
import os
import sys

_HERE = os.path.dirname(os.path.abspath(__file__))
REF_ROOT = os.environ.get("ADRT_REFERENCE_ROOT", "/root/reference")
_cached = None


def _ext_path():
    hits = glob.glob(os.path.join(_HERE, "_ref", "_adrt_cdefs*.so"))
    return hits[0] if hits else None


def load():
    """Return the reference ``adrt`` package, or None when it is unavailable."""
    global _cached
    if _cached is not None:
        return _cached
    src = os.path.join(REF_ROOT, "src", "adrt")
    ext = _ext_path()
    if not os.path.isdir(src) or ext is None:
        return None
    # Load the compiled extension under the name the package expects, then the
    # package itself from the (read-only) checkout.
    loader = importlib.machinery.ExtensionFileLoader("adrt._adrt_cdefs", ext)
    spec = importlib.util.spec_from_file_location("adrt._adrt_cdefs", ext, loader=loader)
    cdefs = importlib.util.module_from_spec(spec)
    loader.exec_module(cdefs)
    saved = sys.modules.get("adrt")
    pkg_spec = importlib.util.spec_from_file_location(
        "adrt", os.path.join(src, "__init__.py"), submodule_search_locations=[src]
    )
    pkg = importlib.util.module_from_spec(pkg_spec)
    sys.modules["adrt"] = pkg
    sys.modules["adrt._adrt_cdefs"] = cdefs
    try:
        pkg_spec.loader.exec_module(pkg)
    except Exception:
        if saved is not None:
            sys.modules["adrt"] = saved
        raise
    _cached = pkg
    return pkg
