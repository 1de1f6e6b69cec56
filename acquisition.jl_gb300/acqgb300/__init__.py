"""acqgb300 — GB300-native FM-DBZP GNSS acquisition (drop-in for Acquisition.jl's acquire path).

The compute runs in hand-written sm_103a CUDA kernels inside ``libacqgb300.so``; this package
is the host-side mirror of the reference's public API (``plan_acquire``, ``acquire!`` spelled
``acquire_b``, ``acquire``, ``AcquisitionResults``, ``is_detected``, ``get_num_cells``,
``cfar_threshold``) over the library's C ABI.
"""
from ._lib import LIB_PATH, load  # noqa: F401
from .api import (AbstractNoiseEstimator, AcquisitionError, AcquisitionPlan, AcquisitionResults,  # noqa: F401
                  ArgumentError, GalileoE1B, GlobalMeanNoiseEstimator, GNSSSystem, GPSL1CA, GPSL5I,
                  OppositeRowNoiseEstimator, acquire, acquire_b, acquire_device, acquire_device_async,
                  cfar_threshold, chip_order, fetch_results, get_num_cells, is_detected, plan_acquire,
                  plan_chip_axis, plan_geometry)

__all__ = ["plan_acquire", "acquire_b", "acquire", "AcquisitionResults", "AcquisitionPlan", "is_detected",
           "get_num_cells", "cfar_threshold", "GPSL1CA", "GPSL5I", "GalileoE1B", "OppositeRowNoiseEstimator",
           "GlobalMeanNoiseEstimator", "AbstractNoiseEstimator", "ArgumentError", "AcquisitionError",
           "acquire_device", "acquire_device_async", "fetch_results", "plan_geometry", "GNSSSystem", "load",
           "chip_order", "plan_chip_axis"]
