"""GB300-native SAR time-domain back-projection focuser.

Drop-in for the focusing call of the reference SAR back-projection project
(``FocalizzatoreBpPx``, sar_focuser_puntual_noui.py:149): Python host code on
PyTorch device tensors calling hand-written sm_103a CUDA kernels through the
C ABI of libsarbp.so (include/sarbp.h).
"""
from ._lib import SarbpError, Tuning, default_tuning, load as load_library
from .focuser import (FocalizzatoreBpCuPy, FocalizzatoreBpCuPy_Batched, FocalizzatoreBpPx,
                      FocusResult, focus, workspace_bytes)
from .scene import DeviceScene, scene_to_device

__all__ = [
    "FocalizzatoreBpPx", "FocalizzatoreBpCuPy", "FocalizzatoreBpCuPy_Batched",
    "focus", "FocusResult", "workspace_bytes", "DeviceScene", "scene_to_device",
    "SarbpError", "Tuning", "default_tuning", "load_library",
]
