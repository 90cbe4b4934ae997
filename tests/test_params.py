"""Configuration handling of the unbinding parameters (Parameter_t subset)."""
import numpy as np
import pytest

from hbtplus_gb300 import synthetic as S
from hbtplus_gb300.unbind import Cosmology, Parameters, params_from_reference

CONF = """#sample config file
[Compulsary Params]
SnapshotPath  /path/to/snapshots
HaloPath /path/to/groups
SubhaloPath /path/to/out
SnapshotFileBase snap_milli   # prefix
MaxSnapshotIndex 63
BoxSize 62.5
SofteningHalo 5e-3
[Optional]
MinNumPartOfSub 30
MaxSampleSizeOfPotentialEstimate 0
TreeNodeOpenAngle 0.7
RefineMostboundParticle 0
LengthInMpch 1e-3
"""


def test_config_file_parsing(tmp_path):
    f = tmp_path / "a.conf"
    f.write_text(CONF)
    p = Parameters.from_config_file(str(f))
    assert p.SofteningHalo == 5e-3 and p.BoxSize == 62.5
    assert p.MinNumPartOfSub == 30 and p.MaxSampleSizeOfPotentialEstimate == 0
    assert p.TreeNodeOpenAngle == 0.7 and p.RefineMostboundParticle is False
    assert p.BoundMassPrecision == 0.995  # default
    # G = 43.0071 (M/1e10) / V^2 / L  (src/config_parser.cpp:95)
    assert p.G == pytest.approx(43007.1, rel=1e-6)
    d = params_from_reference(p, Cosmology.set(1.0, 0.3, 0.7, p.H0))
    assert d["softening"] == 5e-3 and d["hubble"] == pytest.approx(100.0 * 1e-3)


def test_config_rejects_unknown_and_missing(tmp_path):
    f = tmp_path / "b.conf"
    f.write_text(CONF + "NotAKey 3\n")
    with pytest.raises(ValueError, match="unrecognized"):
        Parameters.from_config_file(str(f))
    f.write_text("BoxSize 10\n")
    with pytest.raises(ValueError, match="missing"):
        Parameters.from_config_file(str(f))


def test_cosmology_matches_reference_formula():
    c = Cosmology.set(0.5, 0.3, 0.7)
    hr = np.sqrt(0.3 / 0.125 + 0.0 / 0.25 + 0.7)
    assert c.Hz == pytest.approx(100 * hr, rel=1e-6)


def test_synthetic_batch_sizes_follow_power_law():
    rng = np.random.Generator(np.random.PCG64(1))
    n = S.batch_sizes(rng, 20000)
    assert n.min() >= 20 and n.max() <= 200000
    # dN/dlnN ~ N^-0.9: the fraction above 1000 is about (1000/20)^-0.9
    frac = np.mean(n > 1000)
    assert abs(frac - 50 ** -0.9) < 0.01
