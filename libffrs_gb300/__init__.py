"""libffrs_gb300 -- GB300 (sm_103a) implementation of libffrs's block-coding path.

Importing this package loads the in-tree pybind11 extension ``libffrs`` (built
by ``libffrs_gb300.build``) and registers it under the top-level name
``libffrs``, which is what the reference's pure-Python ``ffrs`` package imports
(``from libffrs import *``).  The extension runs every encode and repair on the
GPU; there is no CPU fallback, so a missing extension raises ImportError here.
"""

import importlib.util
import os
import sys

from . import build as _build

_HERE = os.path.dirname(os.path.abspath(__file__))


def _load():
    path = _build.module_path()
    if not os.path.exists(path):
        raise ImportError(
            f"libffrs_gb300: native extension {os.path.basename(path)} is not built; "
            "run `python -c 'import __graft_entry__ as g; g.build()'`"
        )
    spec = importlib.util.spec_from_file_location("libffrs", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


libffrs = sys.modules.get("libffrs")
if libffrs is None or not getattr(libffrs, "__file__", "").startswith(_HERE):
    libffrs = _load()
    sys.modules["libffrs"] = libffrs

from libffrs import *  # noqa: E402,F401,F403

__all__ = [n for n in dir(libffrs) if not n.startswith("_")]
