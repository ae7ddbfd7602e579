"""The case reader of gb_solver_create, run on the host alone (gb_case_info, no GPU): counts of
blocks, patches, interfaces and mixing planes of the committed cases, the node coordinates parsed
exactly as the reference's stream reads them (compared bit for bit with numpy's parse of the same
text), and the reader's refusals."""
import os
import shutil

import numpy as np
import pytest

from conftest import golden_dir


@pytest.fixture(scope="module")
def built(gbturbo):
    import build as pkg_build
    pkg_build.build()
    return gbturbo


def _grid_nodes(case_dir):
    """x, y, z of every node of the text grid, block after block (the file's own order)"""
    lines = open(os.path.join(case_dir, "grid.dat")).read().split("\n")
    nb, pos, out = int(lines[0]), 1, []
    for _ in range(nb):
        pos += 1                                   # block id
        IM, JM, KM = (int(v) for v in lines[pos].split())
        pos += 1
        n = IM * JM * KM
        out.append(np.array([[float(t) for t in l.split()] for l in lines[pos:pos + n]]))
        pos += n
    return np.concatenate(out)


@pytest.mark.parametrize("name,expect", [
    ("duct_9x9x17", dict(blocks=1, levels=1, inlets=1, outlets=1, interfaces=0, mixing_planes=0)),
    ("rotor_9x9x33_mg", dict(blocks=1, levels=2, inlets=1, outlets=1, interfaces=0, mixing_planes=0)),
    ("rotor_9x9x33_3block", dict(blocks=3, levels=1, inlets=1, outlets=1, interfaces=2, mixing_planes=0)),
    ("stage_9x9x17_mg", dict(blocks=2, levels=2, inlets=1, outlets=1, interfaces=0, mixing_planes=1)),
])
def test_counts_and_nodes(built, name, expect):
    info, xyz = built.case_info(golden_dir(name), nodes=True)
    for k, v in expect.items():
        assert info[k] == v, (k, info[k], v)
    ref = _grid_nodes(golden_dir(name))
    assert info["nodes"] == ref.shape[0]
    assert np.array_equal(xyz, ref)


def _copy_case(name, dst):
    for f in os.listdir(golden_dir(name)):
        shutil.copy(os.path.join(golden_dir(name), f), dst)


def test_patch_naming_a_missing_block_is_refused(built, tmp_path):
    _copy_case("duct_9x9x17", tmp_path)
    bc = (tmp_path / "BoundaryDefinition.dat").read_text().split("\n")
    i = next(n for n, l in enumerate(bc) if "number of inlets" in l) + 2
    f = bc[i].split("\t")
    f[1] = "2"
    bc[i] = "\t".join(f)
    (tmp_path / "BoundaryDefinition.dat").write_text("\n".join(bc))
    with pytest.raises(built.GBError, match="names block 2"):
        built.case_info(str(tmp_path))


def test_mixing_plane_on_other_faces_is_refused(built, tmp_path):
    _copy_case("stage_9x9x17", tmp_path)
    bc = (tmp_path / "BoundaryDefinition.dat").read_text().split("\n")
    i = next(n for n, l in enumerate(bc) if "number of MixingPlanes" in l) + 2
    f = bc[i].split("\t")
    f[3] = "5"                                     # first side on a k- face
    bc[i] = "\t".join(f)
    (tmp_path / "BoundaryDefinition.dat").write_text("\n".join(bc))
    with pytest.raises(built.GBError, match="mixing plane"):
        built.case_info(str(tmp_path))


def test_spalart_allmaras_with_multigrid_is_refused_on_the_host(built, meshgen, tmp_path):
    meshgen.write_case(meshgen.annular_duct(IM=9, JM=9, KM=17, options={"turb": "200", "multigrid": "Y",
                                                                          "coarse_iter": "2"}), str(tmp_path))
    with pytest.raises(built.GBError, match="single grid"):
        built.case_info(str(tmp_path))


def test_short_grid_is_reported(built, tmp_path):
    _copy_case("duct_9x9x17", tmp_path)
    g = (tmp_path / "grid.dat").read_text().split("\n")
    (tmp_path / "grid.dat").write_text("\n".join(g[:200]) + "\n")
    with pytest.raises(built.GBError, match="ended"):
        built.case_info(str(tmp_path))


def test_large_grid_parsed_in_parallel_threads(built, meshgen, tmp_path):
    """a grid of more than 65,536 nodes is parsed by several host threads: every coordinate as the
    one-thread parse gives it, and a bad line reported by its own line number"""
    meshgen.write_case(meshgen.rotor_passage(IM=25, JM=41, KM=97, options={}), str(tmp_path))
    info, xyz = built.case_info(str(tmp_path), nodes=True)
    ref = _grid_nodes(str(tmp_path))
    assert info["nodes"] == ref.shape[0] == 25 * 41 * 97
    assert np.array_equal(xyz, ref)
    g = (tmp_path / "grid.dat").read_text().split("\n")
    bad = 3 + 70000                                # 1-based line of node 70000 (count, id, size lines first)
    g[bad - 1] = "0.1 x 0.3"
    (tmp_path / "grid.dat").write_text("\n".join(g))
    with pytest.raises(built.GBError, match=f"bad node line {bad}$"):
        built.case_info(str(tmp_path))
