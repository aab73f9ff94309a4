"""quasi_gb300: a GB300-native (sm_103a) CUDA rendering backend for the Quasi plugin host.

The product is libquasi_cuda.so (built from quasi_gb300/csrc by quasi_gb300/build.py); this
package is its Python host: ctypes mirrors of the C ABI and a loader that behaves like the
reference's src/quasi/plugin/loader.hpp.
"""
from .host import (DEFAULT_LIBRARY, Batch, LoaderError, PluginHost, QuasiError, Scene, camera_dict, load_library,
                   make_camera, make_scene)

__all__ = ["DEFAULT_LIBRARY", "Batch", "LoaderError", "PluginHost", "QuasiError", "Scene", "camera_dict",
           "load_library", "make_camera", "make_scene"]
