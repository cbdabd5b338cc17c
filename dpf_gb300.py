"""Import name for the package directory ``dynamic-powerfoam_gb300/``.

A hyphen is not valid in a Python module name, so ``import dpf_gb300`` loads
the package from that directory under this name.
"""
import importlib.util
import os
import sys

_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'dynamic-powerfoam_gb300')
_spec = importlib.util.spec_from_file_location(__name__, os.path.join(_DIR, '__init__.py'),
                                               submodule_search_locations=[_DIR])
_module = importlib.util.module_from_spec(_spec)
sys.modules[__name__] = _module
_spec.loader.exec_module(_module)
