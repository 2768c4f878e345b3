"""qubatron_gb300: GB300-native octree ray casting for qubatron.

The compute is libqbcuda (hand-written CUDA for sm_103a behind the C ABI in
include/qbcuda.h); this package is its Python host side:

* ``octree_glc``  mirror of the reference's GL connector API
                  (octree_glc_init / _upload_texbuffer_data / _update)
* ``octree``      the node-array producer of src/qubatron/octree.c
* ``scenes``      seeded synthetic scenes and camera poses
"""
from ._lib import QbcError, View, Outputs, lib_path, load  # noqa: F401
from .octree import Octree, build_octree  # noqa: F401
from .octree_glc import (  # noqa: F401
    GL_FLOAT,
    GL_INT,
    OCTREE_GLC_BUFFER_DYNAMIC_COLOR,
    OCTREE_GLC_BUFFER_DYNAMIC_NORMAL,
    OCTREE_GLC_BUFFER_DYNAMIC_OCTREE,
    OCTREE_GLC_BUFFER_STATIC_COLOR,
    OCTREE_GLC_BUFFER_STATIC_NORMAL,
    OCTREE_GLC_BUFFER_STATIC_OCTREE,
    FrameBuffers,
    OctreeGLC,
    octree_glc_init,
    octree_glc_update,
    octree_glc_upload_texbuffer_data,
    view_setup,
)

__version__ = "0.1.0"
