"""The mixed form against an FP32 hazard of the reference's Roe flux. Its tangential wave strengths
divide a momentum jump by (v + 1e-8) (source/Flux_Split_Scheme.cpp:568-635, the a2 and a3 terms).
FP32 round-off of a near-zero tangential velocity is about 1e-8, so that denominator can reach 0.
Point 9 of the seeded operating-point sampler (back pressure 1.167 x p_t, 12800 rpm, 97 x 41 x 41
nodes) did so on its first full multigrid cycle, and its mixed solve turned NaN. With the
denominator held at half the regularisation, the mixed solve stays finite and follows the FP64
solve."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_sampled_point_with_a_vanishing_roe_denominator(gpu_lib, meshgen, tmp_path):
    op = meshgen.sample_operating_points(64, 2024)[9]
    case = meshgen.rotor_passage(IM=op["IM"], JM=op["JM"], KM=op["KM"], rpm=op["rpm"],
                                 stagger_offset=op["stagger_offset"],
                                 options={"Pout": "%.1f" % (op["pb"] * 101325.0), "multigrid": "Y",
                                          "coarse_iter": "2", "Ma0": "0.45"})
    meshgen.write_case(case, str(tmp_path))
    hist = {}
    for prec in (gpu_lib.MIXED, gpu_lib.FP64):
        with gpu_lib.Solver(str(tmp_path), prec) as s:
            s.init_uniform()
            hist[prec] = s.iterate(20)[:, 0, :]
            assert int(s.status()[0]) & 1 == 0
    a, b = hist[gpu_lib.MIXED], hist[gpu_lib.FP64]
    assert np.all(np.isfinite(a[:, [1, 6, 7, 8, 9]]))
    for col in (6, 7, 8):
        assert float(np.max(np.abs(a[:, col] - b[:, col]) / np.abs(b[:, col]))) < 1e-5
