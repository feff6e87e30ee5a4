from .binary import (
    binary_closing,
    binary_dilation,
    binary_erosion,
    binary_fill_holes,
    binary_hit_or_miss,
    binary_opening,
    binary_propagation,
)
from .grey import (
    black_tophat,
    grey_closing,
    grey_dilation,
    grey_erosion,
    grey_opening,
    morphological_gradient,
    morphological_laplace,
    white_tophat,
)
from .structure import generate_binary_structure, iterate_structure

__all__ = [
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
]
