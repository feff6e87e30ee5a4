"""torchmorph_gb300: GB300-native (sm_103a) drop-in for torchmorph's morphology,
distance-transform and Sinkhorn operators.

``import torchmorph_gb300 as tm`` exposes the reference's public API
(torchmorph/__init__.py) backed by libtmcore.so.
"""

from .distance_transform import (
    brute_force_distance_transform,
    chamfer_distance_transform,
    euclidean_distance_transform,
    euclidean_distance_transform_squared,
)
from .morphology import (
    binary_closing,
    binary_dilation,
    binary_erosion,
    binary_fill_holes,
    binary_hit_or_miss,
    binary_opening,
    binary_propagation,
    black_tophat,
    generate_binary_structure,
    grey_closing,
    grey_dilation,
    grey_erosion,
    grey_opening,
    iterate_structure,
    morphological_gradient,
    morphological_laplace,
    white_tophat,
)
from .optimal_transport import SinkhornSolver, build_cost_matrix
from . import ragged
from .pointcloud_ot import PointCloudSinkhorn, pack_clouds
from .ragged import RaggedBatch

__all__ = [
    "euclidean_distance_transform",
    "euclidean_distance_transform_squared",
    "chamfer_distance_transform",
    "brute_force_distance_transform",
    "generate_binary_structure",
    "iterate_structure",
    "binary_erosion",
    "binary_dilation",
    "binary_fill_holes",
    "binary_hit_or_miss",
    "binary_opening",
    "binary_closing",
    "binary_propagation",
    "grey_erosion",
    "grey_dilation",
    "grey_opening",
    "grey_closing",
    "morphological_gradient",
    "morphological_laplace",
    "white_tophat",
    "black_tophat",
    "SinkhornSolver",
    "build_cost_matrix",
    "ragged",
    "RaggedBatch",
    "PointCloudSinkhorn",
    "pack_clouds",
]
