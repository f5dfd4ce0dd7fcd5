"""Synthetic workloads (shapes, layout, unit of work) and quality metrics."""
import numpy as np
import pytest

from sar_backprojection_gb300 import quality, synth


def test_small_workload_layout():
    sc = synth.generate(synth.config_small())
    assert sc["xxg1"].shape == (256, 64) and sc["xxg1"].flags.f_contiguous
    assert sc["RawData"].shape == (512, 2001) and sc["RawData"].dtype == np.complex64
    assert sc["RawData"].flags.f_contiguous
    assert sc["Index"].dtype == np.int32 and sc["Sint"].dtype == np.int32
    assert sc["Mask"].dtype == np.uint8 and (sc["Mask"] == 1).all()
    assert sc["wgsx"].shape == (2001,)
    # nominal pixel-pulses: 16384 pixels x 401 pulses
    assert synth.nominal_pixel_pulses(sc) == 6_569_984


def test_generation_is_deterministic():
    a = synth.generate(synth.config_small(3))
    b = synth.generate(synth.config_small(3))
    assert synth.input_digest(a) == synth.input_digest(b)
    c = synth.generate(synth.config_small(4))
    assert synth.input_digest(a) != synth.input_digest(c)


def test_full_workload_geometry_only():
    spec = synth.config_full()
    g = synth.geometry(spec)
    assert g["xxg1"].shape == (4000, 250)
    assert g["wgsx"].shape == (40001,)
    assert np.all(np.diff(g["wgsx"]) > 0)
    motion = np.abs(g["wgsy"] + 2000.0).max()
    assert motion <= 1.0 + 1e-9
    assert abs(g["zzg1"].std() - 30.0) < 1e-6
    frac = (g["Mask"] == 1).mean()
    assert 0.79 < frac < 0.81
    assert g["Sint"].min() == 1200 and g["Sint"].max() == 1800
    # every pixel's slant range lands inside the 4762-bin swath
    R = np.sqrt(((g["yyg1"] + 2000.0) ** 2) + (3000.0 - g["zzg1"]) ** 2)
    bins = (R - spec.near_range) / spec.delta_range
    assert bins.min() > 60 and bins.max() < spec.nra - 60


def test_uneven_specs_cover_ranges():
    specs = synth.uneven_specs()
    assert len(specs) == 48
    d0 = [s.dim0 for s in specs]
    nz = [s.naz for s in specs]
    assert min(d0) >= 128 and max(d0) <= 2000
    assert min(nz) >= 2001 and max(nz) <= 20001
    assert all(s.sint_hi <= 1800 and s.sint_lo >= 200 for s in specs)


def test_quality_metrics():
    rng = np.random.default_rng(0)
    b = rng.standard_normal(1000) + 1j * rng.standard_normal(1000)
    assert quality.coherence(b, b) == pytest.approx(1.0)
    assert quality.rel_l2(b, b) == 0.0
    a = b * np.exp(1j * 1e-3)
    st = quality.compare(a, b)
    assert st["rms_phase_mrad"] == pytest.approx(1.0, rel=1e-6)
    assert st["coherence"] == pytest.approx(1.0)
    assert st["phase"]["large_errors"]["pi_32"] == 0
    # float pairs are accepted as complex
    pairs = np.stack([b.real, b.imag], axis=-1)
    assert quality.rel_l2(pairs, b) == 0.0
