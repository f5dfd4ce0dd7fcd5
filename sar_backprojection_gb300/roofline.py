"""Roofline constants of the back-projection path (frozen: bench lines stay comparable).

Unit of work: one nominal pixel-pulse back-projection = one (pixel, pulse)
pair of an unmasked pixel's aperture, ``sum over pixels with mask == 1 and
Sint != -9999 of ceil(Sint/2)*2 + 1`` (implementation independent).

The path is an FP32/SFU issue-bound gather-and-rotate, not an HBM stream and
not a tensor contraction.  Algorithmic operations per pixel-pulse:

* FP32 pipe, N_FP32 = 20: 3 subtractions + 3 FMA for R^2, 1 for the range
  bin, 3 for the phase increment, 4 for the complex rotation, 2 for the R^2
  weight, 2 for the accumulation, 2 miscellaneous;
* SFU, N_SFU = 3: one reciprocal square root (or square root), sin, cos;
* FP64 pipe for the plain FP64 kernel, N_FP64 = 20 (same count, in FP64).

Kahan compensation and range-bin tie re-derivation are not counted.
Peak pixel-pulses/s = min(FP32 FMA lanes/s / N_FP32, SFU ops/s / N_SFU) for
the mixed kernel and FP64 FMA lanes/s / N_FP64 for the FP64 kernel.  The
rates are the larger of two figures: the device's nominal rate (SMs x 128
FP32 lanes, x 16 SFU lanes per clock at the maximum SM clock; GB300's
nominal 1.25 TFLOP/s FP64) and the rate libsarbp's probe kernels measure on
the device, so a fraction never flatters a kernel by a probe that ran slow.

Algorithmic bytes per scene (for the HBM view): the raw-data rows inside the
scene's aperture hull read once (8 B per range bin per pulse), 29 B per DEM
pixel (x, y, z, Index, Sint, Mask), 24 B per trajectory pulse and 16 B per
output pixel.
"""
from __future__ import annotations

N_FP32 = 20
N_SFU = 3
N_FP64 = 20
DEM_BYTES_PER_PIXEL = 8 * 3 + 4 + 4 + 1
TRAJ_BYTES_PER_PULSE = 24
OUT_BYTES_PER_PIXEL = 16
RAW_BYTES_PER_SAMPLE = 8


FP32_LANES_PER_SM_CLK = 128
SFU_LANES_PER_SM_CLK = 16
FP64_FMA_LANES_NOMINAL = 1.25e12 / 2      # GB300: 1.25 TFLOP/s FP64, 2 flops per FMA


def nominal_rates(sms: int, sm_max_mhz: float) -> tuple[float, float, float]:
    """(FP32 FMA lanes/s, SFU ops/s, FP64 FMA lanes/s) of the device on paper."""
    clk = sm_max_mhz * 1e6
    return (sms * FP32_LANES_PER_SM_CLK * clk, sms * SFU_LANES_PER_SM_CLK * clk,
            FP64_FMA_LANES_NOMINAL)


def peak_pixel_pulses(ffma_lanes_per_s: float, sfu_per_s: float) -> float:
    return min(ffma_lanes_per_s / N_FP32, sfu_per_s / N_SFU)


def peak_pixel_pulses_fp64(dfma_lanes_per_s: float) -> float:
    return dfma_lanes_per_s / N_FP64


def algorithmic_bytes(npix: int, naz: int, nra: int, pulses_used: int | None = None) -> int:
    """Bytes a perfect implementation moves once per scene.

    ``pulses_used``: pulses inside the union of apertures (default: all).
    """
    p = naz if pulses_used is None else pulses_used
    return (RAW_BYTES_PER_SAMPLE * nra * p + DEM_BYTES_PER_PIXEL * npix
            + TRAJ_BYTES_PER_PULSE * naz + OUT_BYTES_PER_PIXEL * npix)
