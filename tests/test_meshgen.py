"""Synthetic workload meshes: sizes of every recipe (cells, faces) and basic validity."""
import numpy as np
import pytest

from mycode_gb300 import meshgen as mg


@pytest.mark.parametrize("fn,cells,faces", [
    (mg.wedge, 19_200, 29_000),
    (mg.laminar_plate, 28_800, 57_960),
    (mg.turb_plate, 115_200, 231_120),
])
def test_recipe_sizes(fn, cells, faces):
    s = fn()
    assert s.n_cells == cells and s.expected_faces() == faces


def test_swbli_size():
    s = mg.swbli()
    assert s.n_cells == 768_000 and s.expected_faces() == 1_281_440


@pytest.mark.parametrize("n", [64_000, 256_000])
def test_bump_sizes(n):
    s = mg.bump(n)
    ny = round((n / 6) ** 0.5)
    assert s.n_cells == 2 * 3 * ny * ny


def test_cells_positive_area_and_tags():
    for s in (mg.wedge(), mg.laminar_plate(), mg.bump(20_000), mg.swbli(80, 64)):
        xy = s.nodes
        for c in s.cells[:: max(1, s.n_cells // 500)]:
            k = 3 if c[3] < 0 else 4
            p = xy[c[:k]]
            a = 0.5 * np.sum(p[:, 0] * np.roll(p[:, 1], -1) - np.roll(p[:, 0], -1) * p[:, 1])
            assert a > 0
        assert set(np.unique(s.bedges[:, 2])) <= {1, 2, 3, 4, 5, 6}


def test_plate_first_spacing_and_stretching():
    s = mg.laminar_plate()
    y = np.unique(s.nodes[:, 1])
    h = np.diff(y)
    np.testing.assert_allclose(h[1:] / h[:-1], 1.08, rtol=1e-9)
