"""The mixed form's face stage on tiles staged in shared memory by TMA (cp.async.bulk.tensor), in both
its forms (GBTURBO_FACE_TMA=1: one CTA per tile; =2: persistent CTAs with two buffers), against the
plain face kernel that reads its stencils straight from HBM: all run the same face arithmetic
(face_body.cuh), so the face fluxes and residuals agree to FP32 rounding of the compiler's
instruction choices (bar 1e-6 normwise relative), and so do the histories that follow. Covers a
single passage whose two levels are both staged, a batch of uneven passages in one handle, and the
refusal of meshes the staged forms do not take (the plain kernel then runs)."""
import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu

FIELDS = ["FcI", "FcJ", "FcK", "FvI", "FvJ", "FvK", "res"]


def _rotor(meshgen, d, IM, JM, KM, pb=1.10):
    opts = {"Pout": "%.1f" % (pb * 101325.0), "multigrid": "Y", "coarse_iter": "2", "Ma0": "0.45"}
    meshgen.write_case(meshgen.rotor_passage(IM=IM, JM=JM, KM=KM, options=opts), d)
    return d


def _run(gpu_lib, dirs, monkeypatch, form, cycles):
    monkeypatch.setenv("GBTURBO_FACE_TMA", form)
    s = gpu_lib.Solver(dirs, gpu_lib.MIXED)
    monkeypatch.delenv("GBTURBO_FACE_TMA")
    s.init_uniform()
    h = s.iterate(cycles)
    s.resflux(1)
    return s, h


@pytest.mark.parametrize("form", ["1", "2"])
def test_staged_face_stage_matches_the_plain_kernel(gpu_lib, meshgen, tmp_path, monkeypatch, form):
    d = _rotor(meshgen, str(tmp_path / "r25"), 25, 25, 65)
    a, ha = _run(gpu_lib, [d], monkeypatch, form, 12)
    b, hb = _run(gpu_lib, [d], monkeypatch, "0", 12)
    with a, b:
        assert a.face_staging(1) and a.face_staging(2)
        assert not b.face_staging(1) and not b.face_staging(2)
        for name in FIELDS:
            assert rel_err(a.get(name), b.get(name)) < 1e-6, name
        assert np.all(a.status() == 0)
    cols = [1, 6, 7, 8, 9]
    assert rel_err(ha[:, :, cols], hb[:, :, cols]) < 1e-6


@pytest.mark.parametrize("form", ["1", "2"])
def test_staged_face_stage_in_an_uneven_batch(gpu_lib, meshgen, tmp_path, monkeypatch, form):
    dirs = [_rotor(meshgen, str(tmp_path / "a"), 25, 25, 65, 1.05),
            _rotor(meshgen, str(tmp_path / "b"), 17, 17, 33, 1.15),
            _rotor(meshgen, str(tmp_path / "c"), 41, 41, 97, 1.25)]
    a, ha = _run(gpu_lib, dirs, monkeypatch, form, 8)
    b, hb = _run(gpu_lib, dirs, monkeypatch, "0", 8)
    with a, b:
        assert a.face_staging(1)
        for q in range(3):
            for name in FIELDS:
                assert rel_err(a.get(name, solve=q), b.get(name, solve=q)) < 1e-6, (q, name)
        assert np.all(a.status() == 0)
    assert rel_err(ha[:, :, [1, 6, 7, 8]], hb[:, :, [1, 6, 7, 8]]) < 1e-6


def test_meshes_the_staged_form_does_not_take_run_the_plain_kernel(gpu_lib, meshgen, tmp_path, monkeypatch):
    # KM = 17 (padded k extent 24 < one tile's halo box), KM = 35 (KM + 7 not a multiple of four),
    # IM = JM = 5 (padded extents 12 < the pipelined form's 13-cell halo box)
    monkeypatch.setenv("GBTURBO_FACE_TMA", "2")
    for im, km in ((9, 17), (9, 35), (5, 33)):
        d = str(tmp_path / f"i{im}k{km}")
        opts = {"Pout": "%.1f" % (1.1 * 101325.0), "Ma0": "0.45"}
        meshgen.write_case(meshgen.rotor_passage(IM=im, JM=im, KM=km, options=opts), d)
        with gpu_lib.Solver(d, gpu_lib.MIXED) as s:
            assert not s.face_staging(1)
            s.init_uniform()
            h = s.iterate(3)
            assert np.all(np.isfinite(h[:, :, 1]))
