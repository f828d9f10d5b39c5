"""GB300-native SES mesher: a drop-in for QuickSES's atoms+radii -> SES mesh path.

The compute path is libquickses_gb300.so (hand-written sm_103a CUDA behind a C-ABI that
exports QuickSES's API_* symbols); this package is its Python face.
"""
from .api import (Context, Mesh, QSESError, ReferenceAPI, Server, compute_ses, format_fixed3,  # noqa: F401
                  grid_info, read_pdb, write_obj)
from . import molecules  # noqa: F401

__all__ = ["Context", "Mesh", "QSESError", "ReferenceAPI", "Server", "compute_ses", "format_fixed3", "grid_info", "molecules",
           "read_pdb", "write_obj"]
