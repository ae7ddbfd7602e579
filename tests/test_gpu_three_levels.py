"""The three-level V-cycle extension (gb_solver_create_levels with 3; the reference stops at two
levels, so there is no reference run to compare with): it runs and stays finite on a passage
whose grid coarsens twice, its batches are bit-identical to single solves, the two-level default
is untouched by it, and cases that cannot coarsen twice are refused."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HIST_COLS = [0, 1, 6, 7, 8, 9, 11]


def _rotor(meshgen, path, IM=17, JM=17, KM=65, pb=1.15):
    meshgen.write_case(meshgen.rotor_passage(IM=IM, JM=JM, KM=KM, options={
        "Pout": "%.1f" % (pb * 101325.0), "multigrid": "Y", "coarse_iter": "3", "Ma0": "0.45"}), str(path))
    return str(path)


@pytest.mark.parametrize("prec", ["FP64", "MIXED"])
def test_three_levels_run(gpu_lib, meshgen, tmp_path, prec):
    d = _rotor(meshgen, tmp_path / "c")
    with gpu_lib.Solver(d, getattr(gpu_lib, prec), levels=3) as s:
        assert s.ng == 3
        assert s.dims(0, 3)[:3] == (5, 5, 17)
        s.init_uniform()
        h = s.iterate(40)[:, 0, :]
        assert np.all(np.isfinite(h[:, HIST_COLS]))
        assert int(s.status()[0]) & 1 == 0
        # the three-level cycle moves the state; the mass flows stay physical
        assert h[-1, 6] > 0 and h[-1, 7] > 0


def test_three_level_batch_equals_single_solves(gpu_lib, meshgen, tmp_path):
    a, b = _rotor(meshgen, tmp_path / "a", pb=1.10), _rotor(meshgen, tmp_path / "b", IM=17, JM=21, KM=65, pb=1.20)
    with gpu_lib.Solver([a, b], gpu_lib.FP64, levels=3) as s:
        s.init_uniform()
        hb = s.iterate(10)
    for q, d in enumerate((a, b)):
        with gpu_lib.Solver(d, gpu_lib.FP64, levels=3) as s:
            s.init_uniform()
            h = s.iterate(10)[:, 0, :]
            assert np.array_equal(h[:, HIST_COLS], hb[:, q, HIST_COLS])


def test_two_levels_unchanged_by_the_extension(gpu_lib, meshgen, tmp_path):
    d = _rotor(meshgen, tmp_path / "c")
    out = []
    for levels in (None, 2):
        kw = {} if levels is None else {"levels": levels}
        with gpu_lib.Solver(d, gpu_lib.FP64, **kw) as s:
            assert s.ng == 2
            s.init_uniform()
            out.append(s.iterate(8)[:, 0, HIST_COLS])
    assert np.array_equal(out[0], out[1])


def test_three_levels_refused_where_the_grid_does_not_coarsen_twice(gpu_lib, meshgen, tmp_path):
    d = _rotor(meshgen, tmp_path / "c", IM=9, JM=9, KM=33)          # (9 - 1) / 4 = 2: too coarse
    with pytest.raises(gpu_lib.GBError, match="three grid levels"):
        gpu_lib.Solver(d, gpu_lib.FP64, levels=3)
    meshgen.write_case(meshgen.annular_duct(IM=17, JM=17, KM=33), str(tmp_path / "sg"))   # single grid case
    with pytest.raises(gpu_lib.GBError, match="multigrid"):
        gpu_lib.Solver(str(tmp_path / "sg"), gpu_lib.FP64, levels=3)


def test_three_level_cycle_keeps_the_two_level_converged_state(gpu_lib, meshgen, tmp_path):
    # consistency of the third level's transfers: the converged FP64 state of the two-level FAS
    # (the 25x25x65 rotor at 1.05 x p_t, which meets the reference's rule at cycle 1371) is a fixed
    # point of the three-level V-cycle too, so 60 three-level cycles started from it keep its
    # integrals (a coarse-level correction that did not vanish there would move them). From the
    # uniform start the three-level cycle does not converge on this case (its third level's
    # correction feeds an instability); this pins what it computes, not its convergence.
    d = str(tmp_path / "r")
    meshgen.write_case(meshgen.rotor_passage(IM=25, JM=25, KM=65, options={
        "Pout": "%.1f" % (1.05 * 101325.0), "multigrid": "Y", "coarse_iter": "2", "Ma0": "0.45",
        "maxiter": "6000"}), d)
    with gpu_lib.Solver(d, gpu_lib.FP64) as s:
        s.init_uniform()
        h2 = s.iterate(1400)[:, 0, :]
        cv = s.get("cv")[1:-1, 1:-1, 1:-1]
    assert h2[-1, 1] < 2e-6
    with gpu_lib.Solver(d, gpu_lib.FP64, levels=3) as s:
        assert s.ng == 3
        s.init_uniform()
        s.set_cv(cv)
        s.start_from_fine_state()
        h3 = s.iterate(60)[:, 0, :]
    assert np.all(np.isfinite(h3[:, HIST_COLS]))
    for col in (6, 7, 8):                       # m_in, m_out, PR
        err = float(np.max(np.abs(h3[:, col] - h2[-1, col]) / abs(h2[-1, col])))
        assert err < 1e-4, (col, err)
