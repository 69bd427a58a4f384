"""Import shim: ``import xcore_gb300`` loads the package in ``xcore.jl_gb300/``
(a directory name Python cannot import directly)."""
import importlib.util as _u
import os as _os
import sys as _sys

_pkg = _os.path.join(_os.path.dirname(_os.path.abspath(__file__)), "xcore.jl_gb300")
_spec = _u.spec_from_file_location("xcore_gb300", _os.path.join(_pkg, "__init__.py"),
                                   submodule_search_locations=[_pkg])
_mod = _u.module_from_spec(_spec)
_sys.modules["xcore_gb300"] = _mod
_spec.loader.exec_module(_mod)
