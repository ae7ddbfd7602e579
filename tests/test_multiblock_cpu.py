"""Host side of multi-block cases (no GPU): the axial split of a single-block passage into the
rotor-67 style H-H-H blocks, and the files it writes in the reference's formats."""
import os

import numpy as np

from conftest import golden_dir


def test_axial_split_keeps_nodes_and_cells(meshgen):
    c = meshgen.rotor_passage(IM=9, JM=9, KM=33)
    m = meshgen.split_axial(c, [9, 25])
    assert [b.shape[2] for b in m.blocks] == [9, 17, 9]
    assert m.n_cells == c.n_cells
    # neighbouring blocks share their cut plane
    assert np.array_equal(m.blocks[0][:, :, -1], m.blocks[1][:, :, 0])
    assert np.array_equal(m.blocks[1][:, :, -1], m.blocks[2][:, :, 0])
    assert np.array_equal(np.concatenate([m.blocks[0], m.blocks[1][:, :, 1:], m.blocks[2][:, :, 1:]], axis=2), c.nodes)
    kinds = [(p.patch.kind, p.block, p.block2) for p in m.patches]
    assert ("inlet", 1, 0) in kinds and ("outlet", 3, 0) in kinds
    assert [k for k in kinds if k[0] == "interior"] == [("interior", 1, 2), ("interior", 2, 3)]
    # blade walls only in the middle block, periodic pairs only up- and downstream
    assert {b for kind, b, _ in kinds if kind == "periodic"} == {1, 3}
    blade = [p for p in m.patches if p.patch.kind == "wall" and p.patch.face in (3, 4)]
    assert {p.block for p in blade} == {2}
    # every cell range stays inside its block
    for p in m.patches:
        KM = m.blocks[p.block - 1].shape[2]
        r = p.patch.rng
        assert 1 <= r[4] <= r[5] <= KM


def test_multiblock_fixture_is_the_generator_output(meshgen, tmp_path):
    """the committed case directory of the three-block fixture is what the generator writes"""
    c = meshgen.split_axial(meshgen.rotor_passage(IM=9, JM=9, KM=33, options={}, name="rotor_9x9x33_3block"),
                            [9, 25], name="rotor_9x9x33_3block")
    meshgen.write_multiblock_case(c, str(tmp_path))
    for f in ("config.dat", "BoundaryDefinition.dat", "grid.dat"):
        a = open(os.path.join(golden_dir("rotor_9x9x33_3block"), f)).read()
        b = open(os.path.join(str(tmp_path), f)).read()
        assert a == b, f
    head = open(os.path.join(str(tmp_path), "grid.dat")).read().splitlines()[:3]
    assert head == ["3", "1", "9 9 9"]
