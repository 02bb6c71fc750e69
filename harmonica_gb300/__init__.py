"""
harmonica_gb300: Harmonica's right-rectangular-prism gravity forward model on
NVIDIA GB300 (sm_103a).

Drop-in entry points (same signatures, errors, warnings and units as
harmonica):

* :func:`prism_gravity` -- ``harmonica.prism_gravity``
* :func:`prism_layer` and the ``prism_layer`` accessor
  (:class:`DatasetAccessorPrismLayer`) -- ``harmonica.prism_layer``
* :func:`point_gravity`, :func:`prism_magnetic`, :func:`tesseroid_gravity`,
  :func:`tesseroid_layer` -- the point-mass, magnetic-prism and tesseroid
  forward models

The all-pairs sums run in hand-written CUDA kernels behind the C ABI declared
in ``include/harmonica_gb300.h``; :func:`build` compiles them in-tree.
"""

from ._native import build
from .adjoint import layer_gravity_torch, prism_gravity_torch
from .batch import PrismBatch, autotune, prism_gravity_batch
from .device_layer import DevicePrismLayer, prism_layer_device
from .dipole import dipole_magnetic
from .equivalent_sources import EquivalentSources, EquivalentSourcesSph
from .fields import FIELDS
from .gravity import check_prisms, prism_gravity, prism_gravity_fields
from .layer import DatasetAccessorPrismLayer, PrismLayer, prism_layer
from .magnetic import prism_magnetic
from .magnetic_utils import magnetic_angles_to_vec, magnetic_vec_to_angles, total_field_anomaly
from .point import point_gravity
from .tesseroid import tesseroid_gravity
from .tesseroid_layer import DatasetAccessorTesseroidLayer, TesseroidLayer, tesseroid_layer

__all__ = [
    "DevicePrismLayer",
    "dipole_magnetic",
    "EquivalentSources",
    "EquivalentSourcesSph",
    "prism_layer_device",
    "FIELDS",
    "PrismBatch",
    "autotune",
    "prism_gravity_batch",
    "DatasetAccessorPrismLayer",
    "PrismLayer",
    "build",
    "check_prisms",
    "layer_gravity_torch",
    "prism_gravity_torch",
    "prism_gravity",
    "prism_gravity_fields",
    "prism_layer",
    "point_gravity",
    "prism_magnetic",
    "magnetic_angles_to_vec",
    "magnetic_vec_to_angles",
    "total_field_anomaly",
    "tesseroid_gravity",
    "tesseroid_layer",
    "TesseroidLayer",
    "DatasetAccessorTesseroidLayer",
]
