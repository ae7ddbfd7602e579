"""The CPU oracle against the reference solver's own outputs (tests/golden, made by running the
reference through oracle/_ref). The oracle restates the reference's arithmetic order, so the
match is bit for bit (NaN where the reference divides by a zero momentum component)."""
import numpy as np
import pytest

from conftest import GOLDEN_CASES, golden_dir, load_golden

R1_KEYS = ["cv", "pv", "mut", "omega", "lamcI", "lamcJ", "lamcK", "lamvI", "lamvJ", "lamvK", "dt", "FcI", "FcJ",
           "FcK", "FvI", "FvJ", "FvK", "res", "dIS_pv", "dIP_pv", "dJS_pv", "dJP_pv", "dKS_pv", "dKP_pv", "dIS_cv",
           "dKP_cv"]


def same(a, b):
    return np.array_equal(a, b, equal_nan=True)


# the JST fixtures are checked here against the oracle's restatement of JST_Convective /
# JST_Dissip; the GPU parity tests take them from the reference-only list
JST_CASES = ["duct_9x9x17_jst", "rotor_9x9x33_jst_mg"]


@pytest.mark.parametrize("name", GOLDEN_CASES + JST_CASES)
def test_oracle_bitwise_against_reference(name, oracle_mod):
    g = load_golden(name)
    o = oracle_mod.Oracle(golden_dir(name))
    for key in ("faceI", "faceJ", "faceK", "cell", "totalvol"):
        if "g1_" + key in g:
            assert same(o.get(key), g["g1_" + key]), key
    hist = g["history"]
    mine = o.run(hist.shape[0])
    assert same(mine, hist), "driver history"
    o.resflux(1)
    for key in R1_KEYS:
        if "r1_" + key in g:
            assert same(o.get(key), g["r1_" + key]), key


def test_oracle_reports_bad_case(tmp_path, oracle_mod, meshgen):
    case = meshgen.annular_duct(IM=9, JM=9, KM=17, options={"scheme": "400"})
    meshgen.write_case(case, str(tmp_path))
    with pytest.raises(RuntimeError, match="not on this path"):
        oracle_mod.Oracle(str(tmp_path))


# The oracle's FP32 build (REAL = float) against the reference's own FP32 build: the same operations
# in single precision, so the histories agree to FP32 round-off, not bit for bit (the oracle calls
# the double libm functions where the reference's C++ picks the float overloads). It is the CPU
# timing beside the GPU's mixed form; the tolerance is a few hundred FP32 ulps over the run.
@pytest.mark.parametrize("name", ["duct_9x9x17_fp32", "rotor_9x9x33_mg_fp32"])
def test_oracle_fp32_build_tracks_the_reference_fp32_build(name, oracle_mod):
    g = np.load(golden_dir(name) + ".npz")
    hist = g["history"]
    mine = oracle_mod.Oracle(golden_dir(str(g["case"])), fp32=True).run(hist.shape[0])
    cols = [1, 6, 7, 8]                         # Res.dens, m_in, m_out, PR
    rel = np.abs(mine[:, cols] - hist[:, cols]) / np.abs(hist[:, cols])
    assert rel.max() < 2e-5, rel.max(axis=0)
