"""Loader for the reference adrt package installed in baseline/_ref.

TEST AND BASELINE INFRASTRUCTURE ONLY.  ``make -C oracle install-ref
REF_SRC=<adrt checkout>`` installs the reference package (its Python modules
and C++ sources) into the git-ignored ``baseline/_ref/adrt`` and compiles its
CPython extension there; ``make -C oracle ref`` recompiles the extension on a
host of another architecture.  This module imports that package unmodified,
so callers use the reference's own public API (``adrt.adrt`` and so on).
``ADRT_REFERENCE_INSTALL`` overrides the install directory.  Returns None
where the package or its compiled extension is absent; callers handle that.
"""

from __future__ import annotations

import glob
import importlib.util
import os
import sys

_HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.environ.get("ADRT_REFERENCE_INSTALL", os.path.join(os.path.dirname(_HERE), "baseline", "_ref"))
_cached = None


def available() -> bool:
    pkg = os.path.join(REF_DIR, "adrt")
    return os.path.isfile(os.path.join(pkg, "__init__.py")) and bool(glob.glob(os.path.join(pkg, "_adrt_cdefs*.so")))


def load():
    """Return the reference ``adrt`` package, or None when it is unavailable."""
    global _cached
    if _cached is not None:
        return _cached
    if not available():
        return None
    pkg_dir = os.path.join(REF_DIR, "adrt")
    saved = {k: sys.modules[k] for k in list(sys.modules) if k == "adrt" or k.startswith("adrt.")}
    spec = importlib.util.spec_from_file_location(
        "adrt", os.path.join(pkg_dir, "__init__.py"), submodule_search_locations=[pkg_dir]
    )
    pkg = importlib.util.module_from_spec(spec)
    sys.modules["adrt"] = pkg
    try:
        spec.loader.exec_module(pkg)
    except Exception:
        for k in [k for k in sys.modules if k == "adrt" or k.startswith("adrt.")]:
            del sys.modules[k]
        sys.modules.update(saved)
        raise
    _cached = pkg
    return pkg
