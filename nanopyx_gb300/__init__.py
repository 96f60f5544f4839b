"""GB300-native (sm_103a) eSRRF / SRRF engine with NanoPyx's call surface.

Every computation runs in the CUDA library ``_lib/libnanopyx_gb300.so``
(C ABI: ``include/nanopyx_gb300.h``); there is no CPU fallback.
"""
from ._device import check_image
from ._native import DeviceTimeoutError, NativeLibraryError
from .liquid import LiquidEngine
from .methods import (SRRF, ESRRFAccumulator, Workflow, eSRRF, eSRRF3D, esrrf_device,
                      esrrf_parameter_sweep)
from .scoring import (DecorrAnalysis, ErrorMap, FIRECalculator, ParameterSweep,
                      calculate_decorr_analysis, calculate_error_map, calculate_frc,
                      run_esrrf_parameter_sweep)
from .transform import (CRShiftAndMagnify, GradientRobertsCross, RadialGradientConvergence,
                        Radiality, ShiftAndMagnify, calculate_eSRRF_temporal_correlations,
                        calculate_SRRF_temporal_correlations, eSRRF3D_ST, eSRRF_ST,
                        fht_space_interpolation,
                        macro_pixel_corrector, value2array)

__version__ = "0.1.0"

__all__ = [
    "eSRRF", "SRRF", "eSRRF_ST", "eSRRF3D", "eSRRF3D_ST", "Workflow", "ESRRFAccumulator", "esrrf_device", "esrrf_parameter_sweep",
    "run_esrrf_parameter_sweep", "ShiftAndMagnify", "CRShiftAndMagnify", "GradientRobertsCross",
    "RadialGradientConvergence", "Radiality", "calculate_eSRRF_temporal_correlations",
    "calculate_SRRF_temporal_correlations", "macro_pixel_corrector", "check_image",
    "value2array", "fht_space_interpolation", "LiquidEngine", "NativeLibraryError",
    "DeviceTimeoutError", "ErrorMap", "FIRECalculator", "ParameterSweep", "calculate_error_map",
    "calculate_frc", "DecorrAnalysis", "calculate_decorr_analysis",
]
