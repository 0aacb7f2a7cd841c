"""plumed2_gb300 -- PLUMED's COORDINATION collective variable on GB300 (sm_103a).

The compute lives in libcoordgpu.so (C ABI: include/coordgpu.h).  This
package holds the host-side mirror of the reference's action interface
(``Coordination``), the ctypes binding, the torch autograd binding, the build
script and the synthetic frame generators.
"""
from .frames import jittered_lattice, sc_sites  # noqa: F401


def __getattr__(name):
    if name == "Coordination":
        from .action import Coordination
        return Coordination
    if name == "CoordError":
        from ._lib import CoordError
        return CoordError
    raise AttributeError(name)
