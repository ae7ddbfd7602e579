"""The reference's solution files through the C-ABI, against files the reference itself wrote
(fixture rotor_9x9x33_restart, made by tests/golden/make_golden.py):

- after 10 iterations the GPU writes RestartSolution.dat and RelativeSolution.plt in the
  reference's formats; both hold numbers printed to six significant digits, so they are compared
  number by number at 1.5e-5 relative (a last-digit difference), integers exactly;
- a case whose config asks for the previous solution starts from the reference's
  RestartSolution.dat and runs 10 more iterations; its history and final state match the
  reference's restarted run at the usual 1e-9 / 1e-10."""
import numpy as np
import pytest

from conftest import golden_dir, load_golden, rel_err

pytestmark = pytest.mark.gpu

HIST_COLS = [0, 1, 6, 7, 8, 9, 11]
RTOL_TEXT = 1.5e-5


def _tokens(text: bytes):
    lines = text.decode().splitlines()
    head = [l for l in lines if not l[:1].isdigit() and not l[:1] == "-"]
    nums = [float(t) for l in lines if l[:1].isdigit() or l[:1] == "-" for t in l.split()]
    return head, np.array(nums), lines


def _compare_text(got: bytes, ref: bytes):
    hg, ng, lg = _tokens(got)
    hr, nr, lr = _tokens(ref)
    assert hg == hr
    assert ng.shape == nr.shape
    scale = np.maximum(np.abs(nr), 1e-12 * np.max(np.abs(nr)))
    err = np.abs(ng - nr) / scale
    assert float(err.max()) <= RTOL_TEXT, float(err.max())
    same = sum(a == b for a, b in zip(lg, lr)) / len(lr)
    return same


def test_written_files_match_the_reference(gpu_lib, tmp_path):
    g = load_golden("rotor_9x9x33_restart")
    with gpu_lib.Solver(golden_dir("rotor_9x9x33_restart"), gpu_lib.FP64) as s:
        s.init_uniform()
        h = s.iterate(g["history1"].shape[0])[:, 0, :]
        ref = g["history1"]
        assert np.max(np.abs(h[:, HIST_COLS] - ref[:, HIST_COLS]) / np.abs(ref[:, HIST_COLS])) < 1e-9
        s.write_restart(0, str(tmp_path / "RestartSolution.dat"))
        s.write_solution(0, str(tmp_path / "RelativeSolution.plt"))
    same_r = _compare_text((tmp_path / "RestartSolution.dat").read_bytes(), g["restart_file"].tobytes())
    same_s = _compare_text((tmp_path / "RelativeSolution.plt").read_bytes(), g["solution_file"].tobytes())
    # the states agree to ~1e-12, so almost every line prints identically
    assert same_r > 0.98 and same_s > 0.98, (same_r, same_s)


def test_restart_continues_like_the_reference(gpu_lib):
    g = load_golden("rotor_9x9x33_restart")
    with gpu_lib.Solver(golden_dir("rotor_9x9x33_restart_reuse"), gpu_lib.FP64) as s:
        s.read_restart(0)                       # RestartSolution.dat of the case directory
        h = s.iterate(g["history2"].shape[0])[:, 0, :]
        ref = g["history2"]
        assert np.max(np.abs(h[:, HIST_COLS] - ref[:, HIST_COLS]) / np.abs(ref[:, HIST_COLS])) < 1e-9
        cv = s.get("cv")
        assert rel_err(cv[1:-1, 1:-1, 1:-1], g["s1_cv"][1:-1, 1:-1, 1:-1]) < 1e-10


def test_restart_of_the_mixed_form_runs(gpu_lib):
    with gpu_lib.Solver(golden_dir("rotor_9x9x33_restart_reuse"), gpu_lib.MIXED) as s:
        s.read_restart(0)
        h = s.iterate(5)[:, 0, :]
        assert np.all(np.isfinite(h[:, HIST_COLS]))
        assert int(s.status()[0]) == 0


def test_short_restart_file_is_reported(gpu_lib, tmp_path):
    src = (golden_dir("rotor_9x9x33_restart_reuse") + "/RestartSolution.dat")
    lines = open(src).read().splitlines()
    bad = tmp_path / "short.dat"
    bad.write_text("\n".join(lines[:100]) + "\n")
    with gpu_lib.Solver(golden_dir("rotor_9x9x33_restart_reuse"), gpu_lib.FP64) as s:
        with pytest.raises(gpu_lib.GBError, match="short"):
            s.read_restart(0, str(bad))
