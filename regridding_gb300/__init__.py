"""GB300-native regridding: a drop-in for the conservative and multilinear hot
path of sun-data/regridding, computed by hand-written sm_103a CUDA kernels.

Public functions keep the upstream signatures and the saved-weights layout:
:func:`weights`, :func:`regrid_from_weights`, :func:`regrid`,
:func:`transpose_weights`, :func:`transpose_weights_conservative`,
:func:`find_indices`, :func:`ndarray_linear_interpolation`, :func:`fill`.  :class:`DeviceWeights` exposes the device-resident
matrix for callers that keep their arrays on the GPU.
"""

from ._find_indices import find_indices, locate_2d
from ._interp import ndarray_linear_interpolation
from ._fill import fill
from ._weights import weights
from ._transposed import transpose_weights, transpose_weights_conservative, cell_volume
from ._regrid import regrid_from_weights, regrid
from ._device import DeviceWeights, build_conservative_2d
from ._lib import RegridError

__all__ = [
    "find_indices",
    "ndarray_linear_interpolation",
    "fill",
    "weights",
    "transpose_weights",
    "transpose_weights_conservative",
    "regrid_from_weights",
    "regrid",
    "DeviceWeights",
    "build_conservative_2d",
    "locate_2d",
    "cell_volume",
    "RegridError",
]
