"""GB300-native isosurface-to-image path behind Contour3D's C API.

The product is the native library contour3d_gb300/_build/libcontour3d_gb300.so
(hand-written sm_103a CUDA + C++ host runtime).  This package is its Python
face: ctypes bindings that mirror the reference's `contour3d_execute`
(reference include/contour3d.h:58-86) plus the extensions declared in
include/contour3d_gb300.h.  There is no CPU fallback: every call goes to the
native library, and loading fails loudly when it is missing.
"""
from .lib import Library, load, NativeLibraryMissing  # noqa: F401
from . import _abi  # noqa: F401
