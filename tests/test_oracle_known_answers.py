"""Known-answer vectors of the upstream test-suite, run against the oracle.

Inputs and expected values follow the upstream tests they name
(tests/test_algorithms/*.py, tests/test_celltree.py, tests/test_geometry_utils.py,
tests/test_edgecelltree.py, tests/test_celltree_utils.py)."""

import numpy as np
import pytest

TOL = 1e-9
BOX = (0.0, 2.0, 0.0, 2.0)
POLY = np.array([[0.0, 0.0], [2.0, 0.0], [2.0, 2.0], [0.0, 2.0]])


def _clippers(oracle):
    return [
        ("cs", lambda a, b, box: oracle.cohen_sutherland_line_box_clip(a, b, box), BOX),
        ("lb", lambda a, b, box: oracle.liang_barsky_line_box_clip(a, b, box), BOX),
        ("cb", lambda a, b, poly: oracle.cyrus_beck_line_polygon_clip(a, b, poly, TOL), POLY),
        ("cb_rev", lambda a, b, poly: oracle.cyrus_beck_line_polygon_clip(a, b, poly, TOL), POLY[::-1]),
    ]


# test_line_box_clip.py:47-119
LINE_BOX_CASES = [
    ((-1.0, 0.0), (2.0, 3.0), True, (0.0, 1.0), (1.0, 2.0)),
    ((0.0, -0.1), (0.0, -0.1), False, (np.nan, np.nan), (np.nan, np.nan)),
    ((-1.0, 1.0), (3.0, 1.0), True, (0.0, 1.0), (2.0, 1.0)),
    ((1.0, -3.0), (1.0, 3.0), True, (1.0, 0.0), (1.0, 2.0)),
    ((1.0, -3.0), (1.0, 1.0), True, (1.0, 0.0), (1.0, 1.0)),
    ((1.0, 1.0), (1.0, 3.0), True, (1.0, 1.0), (1.0, 2.0)),
    ((-1.0, 3.0), (3.0, 3.0), False, None, None),
    ((-1.0, 1.0), (1.0, 1.0), True, (0.0, 1.0), (1.0, 1.0)),
    ((0.5, 0.5), (1.5, 1.5), True, (0.5, 0.5), (1.5, 1.5)),
    ((-1.5, 0.0), (-0.5, 1.0), False, None, None),
    ((2.5, 0.0), (3.5, 1.0), False, None, None),
]

# test_line_box_clip.py:131-304 (degeneracies)
DEGENERATE_CASES = [
    ((-1.0, -1.0), (3.0, 3.0), True, (0.0, 0.0), (2.0, 2.0)),
    ((-1.0, -1.0), (-1.0, -1.0), False, (np.nan, np.nan), (np.nan, np.nan)),
    ((-1.0, 0.0), (3.0, 0.0), True, (0.0, 0.0), (2.0, 0.0)),
    ((-1.0, 2.0), (3.0, 2.0), True, (0.0, 2.0), (2.0, 2.0)),
    ((-1.0, 0.0), (1.0, 0.0), True, (0.0, 0.0), (1.0, 0.0)),
    ((-1.0, 2.0), (1.0, 2.0), True, (0.0, 2.0), (1.0, 2.0)),
    ((0.5, 0.0), (1.5, 0.0), True, (0.5, 0.0), (1.5, 0.0)),
    ((0.5, 2.0), (1.5, 2.0), True, (0.5, 2.0), (1.5, 2.0)),
    ((0.0, 0.0), (2.0, 0.0), True, (0.0, 0.0), (2.0, 0.0)),
    ((0.0, 2.0), (2.0, 2.0), True, (0.0, 2.0), (2.0, 2.0)),
    ((0.0, 0.0), (0.0, 2.0), True, (0.0, 0.0), (0.0, 2.0)),
    ((2.0, 0.0), (2.0, 2.0), True, (2.0, 0.0), (2.0, 2.0)),
    ((0.0, 0.5), (0.0, 1.5), True, (0.0, 0.5), (0.0, 1.5)),
    ((2.0, 0.5), (2.0, 1.5), True, (2.0, 0.5), (2.0, 1.5)),
    ((-1.0, 1.0), (0.0, 2.0), False, (np.nan, np.nan), (np.nan, np.nan)),
]


@pytest.mark.parametrize("k", range(3))
@pytest.mark.parametrize("case", LINE_BOX_CASES)
def test_line_box_clip(oracle, k, case):
    name, clip, box = _clippers(oracle)[k]
    a, b, inter, c, d = case
    got, gc, gd = clip(a, b, box)
    assert got is inter
    if c is not None:
        assert np.allclose(gc, c, equal_nan=True)
        assert np.allclose(gd, d, equal_nan=True)


@pytest.mark.parametrize("k", range(4))
@pytest.mark.parametrize("case", DEGENERATE_CASES)
def test_line_box_clip_degeneracy(oracle, k, case):
    name, clip, box = _clippers(oracle)[k]
    a, b, inter, c, d = case
    got, gc, gd = clip(a, b, box)
    assert got is inter
    assert np.allclose(gc, c, equal_nan=True)
    assert np.allclose(gd, d, equal_nan=True)


def test_line_polygon_clip(oracle):
    # test_line_polygon_clip.py:21-102
    clip = lambda a, b, p: oracle.cyrus_beck_line_polygon_clip(a, b, p, TOL)  # noqa: E731
    poly = np.array([[1.0, 3.0], [4.0, 3.0], [4.0, 5.0], [1.0, 5.0]])
    r = clip((0.0, 0.0), (4.0, 6.0), poly)
    assert r[0] and np.allclose(r[1], [2.0, 3.0]) and np.allclose(r[2], [3.3333333333333, 5.0])
    rr = clip((4.0, 6.0), (0.0, 0.0), poly)
    assert r == (rr[0], rr[2], rr[1])
    assert not clip((0.0, 0.1), (0.0, 0.1), poly)[0]
    r = clip((0.0, 4.0), (5.0, 4.0), poly)
    assert r[0] and np.allclose(r[1], [1.0, 4.0]) and np.allclose(r[2], [4.0, 4.0])
    # through vertex
    r = clip((2.0, 2.0), (1.0, 4.0), np.array([[2.0, 4.0], [1.0, 4.0], [1.0, 3.0], [2.0, 3.0]]))
    assert r[0] and np.allclose(r[1], [1.5, 3.0]) and np.allclose(r[2], [1.0, 4.0])
    assert not clip((2.0, 0.0), (2.0, 2.0), np.array([[2.0, 3.0], [1.0, 3.0], [1.0, 2.0], [2.0, 2.0]]))[0]
    assert not clip((2.0, 0.0), (2.0, 2.0), np.array([[3.0, 3.0], [2.0, 3.0], [2.0, 2.0], [3.0, 2.0]]))[0]
    # triangle
    tri = np.array([[0.0, 0.5], [2.0, 0.0], [2.0, 2.0]])
    r = clip((1.0, 1.0), (3.0, 1.0), tri)
    assert r[0] and np.allclose(r[1], [1.0, 1.0]) and np.allclose(r[2], [2.0, 1.0])
    tri = np.array([[0.0, 0.0], [2.0, 0.0], [2.0, 2.0]])
    for a, b in [((0.0, 0.0), (2.0, 0.0)), ((2.0, 0.0), (2.0, 2.0)), ((0.0, 0.0), (2.0, 2.0)),
                 ((-1.0, -1.0), (2.0, 2.0)), ((-1.0, -1.0), (3.0, 3.0)), ((0.0, 0.0), (3.0, 3.0))]:
        assert clip(a, b, tri)[0]
        assert clip(b, a, tri)[0]
    # box degeneracies test_line_polygon_clip.py:171-215
    nodes = np.array([[0.0, 0.0], [1.0, 0.0], [2.0, 0.0], [0.0, 1.0], [1.0, 1.0], [2.0, 1.0], [0.0, 2.0],
                      [1.0, 2.0], [2.0, 2.0]])
    faces = np.array([[3, 4, 6, 7], [4, 5, 8, 7], [0, 1, 4, 3], [1, 2, 5, 4]])
    r = clip((1.0, 1.0), (1.5, 1.25), nodes[faces[1]])
    assert r[0] and r[1] == (1.0, 1.0) and r[2] == (1.5, 1.25)
    for i in [0, 2, 3]:
        assert not clip((1.0, 1.0), (1.5, 1.25), nodes[faces[i]])[0]
    r = clip((0.5, 0.75), (1.0, 1.0), nodes[faces[2]])
    assert r[0] and r[1] == (0.5, 0.75) and r[2] == (1.0, 1.0)


def test_separating_axes(oracle):
    # test_separating_axis.py:9-142
    s = oracle.separating_axes
    a = np.array([[0.0, 0.0], [0.0, 1.0], [1.0, 1.0]])
    assert s(a, a) and s(a, a)
    b = np.array([[2.0, 0.0], [3.0, 1.0], [2.0, 1.0]])
    assert not s(a, b) and not s(b, a)
    b = np.array([[1.0, 0.0], [2.0, 1.0], [1.0, 1.0]])
    assert not s(a, b) and not s(b, a)
    a = np.array([[0.0, 0.0], [4.0, 0.0], [0.0, 4.0]])
    b = np.array([[1.0, 1.0], [2.0, 1.0], [1.0, 2.0]])
    assert s(a, b) and s(b, a)
    a = np.array([[0.0, 0.0], [1.0, 0.0], [0.0, 1.0]])
    b = np.array([[1.0, 0.0], [2.0, 0.0], [2.0, 1.0]])
    assert not s(a, b) and not s(b, a)
    a = np.array([[5.0, 3.0], [7.0, 3.0], [7.0, 5.0]])
    b = np.array([[6.9, 5.6], [8.0, 4.75], [7.85, 5.9]])
    assert s(a, b) and not s(b, a)
    a = np.array([[0.0, 0.0], [2.0, 0.0], [2.0, 2.0], [0.0, 2.0]])
    b = np.array([[1.0, 1.0], [3.0, 0.0], [3.0, 1.0]])
    assert s(a, b) and s(b, a)
    b = np.array([[2.0, 1.0], [3.0, 0.0], [3.0, 1.0]])
    assert not s(a, b) and not s(b, a)
    b = np.array([[0.25, 0.25], [0.75, 0.75], [0.6, 0.6]])
    assert s(a, b) and s(b, a)
    # hanging nodes test_separating_axis.py:185-223
    a = np.array([[0.0, 0.0], [0.5, 0.5], [0.0, 1.0], [1.0, 1.0]])
    assert s(a, a)
    b = np.array([[2.0, 0.0], [3.0, 1.0], [2.5, 1.0], [2.0, 1.0]])
    assert not s(a, b) and not s(b, a)
    a = np.array([[0.0, 0.0], [0.5, 0.5], [0.5, 0.5], [0.0, 1.0], [1.0, 1.0]])
    assert s(a, a)


# test_sutherland_hodgman.py:46-90
SH_A = np.array([
    [[0.98599114, 0.16203056], [0.64839124, 0.6552714], [0.44528724, 0.88567472]],
    [[0.96182162, 0.3642742], [0.03478739, 0.54268026], [0.57582971, 0.41541277]],
    [[0.32556365, 0.03800701], [0.74000686, 0.04684465], [0.89527188, 0.55061165]],
    [[0.2988294, 0.96608896], [0.01212383, 0.00144037], [0.75113002, 0.54797261]],
    [[0.06522962, 0.43735202], [0.791499, 0.5229509], [0.40651803, 0.94317979]],
    [[0.06544202, 0.16735701], [0.67916353, 0.95843272], [0.33545733, 0.86368003]],
    [[0.43129575, 0.27998206], [0.49468229, 0.75438255], [0.01542992, 0.80696797]],
    [[0.29449023, 0.32433138], [0.46157048, 0.22492393], [0.82442969, 0.75853821]],
    [[0.66113797, 0.88485505], [0.70164374, 0.24393423], [0.89565423, 0.89407158]],
    [[0.92226655, 0.82771688], [0.42243438, 0.17562404], [0.82885357, 0.17541439]],
])
SH_B = np.array([
    [[0.8141854, 0.06821897], [0.37086004, 0.49067617], [0.79810508, 0.07873283]],
    [[0.74948185, 0.8942076], [0.59654411, 0.87755533], [0.3023107, 0.68256513]],
    [[0.46670989, 0.31716127], [0.68408985, 0.75792215], [0.41437824, 0.79509823]],
    [[0.60715923, 0.67648133], [0.40045464, 0.79676831], [0.06332723, 0.69679141]],
    [[0.24057248, 0.16433727], [0.58871277, 0.05499277], [0.59144784, 0.24476056]],
    [[0.23183198, 0.41619006], [0.66566902, 0.30110111], [0.60418791, 0.60702136]],
    [[0.09393344, 0.87976118], [0.994083, 0.00532686], [0.95176396, 0.79836557]],
    [[0.89063751, 0.5880825], [0.03881315, 0.82436939], [0.61391092, 0.45027842]],
    [[0.63168954, 0.75135847], [0.8726944, 0.06387274], [0.89585471, 0.92837592]],
    [[0.94379596, 0.64164962], [0.95787609, 0.65627618], [0.6212529, 0.89153053]],
])
SH_EXPECTED = np.array([0.0, 0.0, 0.0, 0.0262324, 0.0, 0.00038042, 0.03629781, 0.01677156, 0.05417924, 0.00108787])


def test_clip_area(oracle):
    for a, b, e in zip(SH_A, SH_B, SH_EXPECTED):
        assert np.allclose(oracle.polygon_polygon_clip_area(a, b), e)
    a = np.array([[0.0, 0.0], [1.0, 0.0], [1.0, 1.0]])
    assert np.allclose(oracle.polygon_polygon_clip_area(a, a + 2.0), 0.0)
    a = np.array([[0.0, 0.0], [1.0, 0.0], [1.0, 0.0], [1.0, 1.0]])
    assert np.allclose(oracle.polygon_polygon_clip_area(a, a + 2.0), 0.0)
    eps = np.finfo(np.float64).eps
    a = np.array([[-1.0, -1.0], [1.0, -1.0], [1.0, 1.0]])
    for e in (eps, -eps):
        b = np.array([[-1.0 - e, -1.0 - e], [1.0 + e, -1.0 - e], [1.0 + e, 1.0 + e]])
        assert np.allclose(oracle.polygon_polygon_clip_area(a, b), 2.0)


def test_polygon_area(oracle):
    # test_geometry_utils.py:95-127
    assert np.allclose(oracle.polygon_area(np.array([[0.0, 0.0], [1.0, 0.0], [1.0, 1.0], [0.0, 1.0]])), 1.0)
    assert np.allclose(oracle.polygon_area(np.array([[0.0, 0.0], [1.0, 0.0], [1.0, 1.0]])), 0.5)
    p = np.array([[0.0, 0.0], [1.0, 0.0], [1.0, 1.0], [0.5, 2.0], [0.0, 1.0]])
    assert np.allclose(oracle.polygon_area(p), 1.5)
    assert np.allclose(oracle.polygon_area(p[::-1]), 1.5)


def test_wachspress(oracle):
    # test_barycentric.py:129-147
    poly = np.array([[0.0, 0.0], [1.0, 0.0], [1.0, 1.0], [0.0, 1.0]])
    cases = [((0.0, 0.0), [1, 0, 0, 0]), ((1.0, 0.0), [0, 1, 0, 0]), ((1.0, 1.0), [0, 0, 1, 0]),
             ((0.0, 1.0), [0, 0, 0, 1]), ((0.25, 0.0), [0.75, 0.25, 0, 0]), ((0.25, 1.0), [0, 0, 0.25, 0.75]),
             ((0.5, 0.5), [0.25, 0.25, 0.25, 0.25])]
    for p, e in cases:
        assert np.allclose(oracle.wachspress_weights(poly, p, 4, TOL), e)


def test_points_in_triangles(oracle):
    # test_geometry_utils.py:439-473
    v = np.array([[0.0, 0.0], [1.0, 0.0], [1.0, 1.0], [2.0, 0.0]])
    f = np.array([[0, 1, 2], [1, 3, 2]])
    pts = np.array([[-0.5, 0.25], [0.0, 0.0], [0.5, 0.5], [0.5, 0.25], [1.5, 0.25], [2.5, 0.25]])
    got = oracle.points_in_triangles(pts, np.array([0, 0, 0, 0, 1, 1]), f, v, 1e-9)
    assert np.array_equal(got, [False, True, True, True, True, False])


NODES2 = np.array([[0.0, 0.0], [2.0, 0.0], [1.0, 2.0], [3.0, 2.0]])
FACES2 = np.array([[0, 1, 2], [1, 3, 2]])


def test_celltree_lookups(oracle):
    # test_celltree.py:167-330
    T = oracle.OracleCellTree2d
    t = T(NODES2, FACES2, -1)
    assert np.array_equal(t.locate_points(np.array([[1.0, 1.0], [2.0, 1.0], [-1.0, 1.0]])), [0, 1, -1])
    pts = np.array([[-0.09, 0.0], [2.0, 1.0], [-1.0, 1.0]])
    assert np.array_equal(t.locate_points(pts, tolerance=1e-9), [-1, 1, -1])
    assert np.array_equal(t.locate_points(pts, tolerance=1e-1), [0, 1, -1])
    nodes = np.array([[0.0, 0.0], [0.0, 2.0], [2.0, 0.0], [2.0, 2.0], [4.0, 0.0], [4.0, 2.0], [6.0, 0.0],
                      [6.0, 2.0], [0.0, 4.0], [2.0, 4.0], [4.0, 4.0], [6.0, 4.0]])
    faces = np.array([[0, 8, 9, 5, 2], [9, 11, 7, 5, -1], [4, 7, 6, -1, -1]])
    t = T(nodes, faces, -1, n_buckets=2, cells_per_leaf=1)
    assert np.array_equal(t.locate_points(np.array([[1.0, 1.0], [5.0, 0.5], [5.0, 3.0], [-1.0, 1.0]])),
                          [0, 2, 1, -1])
    pts = np.array([[-9e-9, 0.0], [2.0, -9e-9], [-9e-9, 1.0], [1.0, -9e-9], [-1.1e-8, 1.0], [1.0, -1.1e-8],
                    [-1.1e-8, 0.0], [2.0, -1.5e-8]])
    assert np.array_equal(t.locate_points(pts), [-1] * 8)
    assert np.array_equal(t.locate_points(pts, tolerance=1e-8), [0, 0, 0, 0, -1, -1, -1, -1])
    bi, bj = t.locate_boxes(np.array([[1.0, 2.0, 1.0, 2.0], [4.0, 5.0, 0.0, 1.0], [4.0, 5.0, 2.0, 3.0],
                                      [-1.0, 0.0, 0.0, 4.0], [6.0, 8.0, 0.0, 4.0], [0.0, 6.0, -1.0, 0.0],
                                      [0.0, 6.0, 4.0, 5.0]]))
    assert np.array_equal(bi, [0, 1, 2]) and np.array_equal(bj, [0, 2, 1])
    edges = np.array([[[1.0, 1.0], [2.0, 2.0]], [[4.0, 3.0], [5.0, 4.0]], [[5.0, 0.0], [6.0, 1.0]],
                      [[-2.0, -1.0], [0.0, 1.0]], [[-2.0, -1.0], [-2.0, -1.0]]])
    i, j, xy = t.intersect_edges(edges)
    assert np.array_equal(i, [0, 1, 2]) and np.array_equal(j, [0, 1, 2]) and np.allclose(xy, edges[:3])
    i, j, xy = t.intersect_edges(edges[:, ::-1])
    assert np.array_equal(i, [0, 1, 2]) and np.allclose(xy, edges[:3, ::-1])
    # test_multipoint test_celltree.py:316-330
    n21 = [(5, 1), (10, 1), (3, 3), (7, 3), (9, 4), (12, 4), (5, 5), (3, 7), (5, 7), (7, 7), (9, 7), (11, 7),
           (5, 9), (8, 9), (11, 9), (9, 11), (11, 11), (7, 13), (9, 13), (7, 15)]
    f21 = [(0, 1, 3), (0, 2, 6), (0, 3, 6), (1, 3, 4), (1, 4, 5), (2, 6, 7), (6, 7, 8), (7, 8, 12), (6, 8, 9),
           (8, 9, 12), (9, 12, 13), (4, 5, 11), (4, 10, 11), (9, 10, 13), (10, 11, 14), (10, 13, 14),
           (13, 14, 15), (14, 15, 16), (15, 16, 18), (15, 17, 18), (17, 18, 19)]
    t = T(n21, f21, -1)
    pts = [(4.2, 3.0), (7.7, 13.5), (3.4, 7.000000001), (7.0, 5.0), (8.66, 10.99), (7.3, 0.74), (2.5, 5.5),
           (9.8, 12.3)]
    assert np.array_equal(t.locate_points(pts), (1, 20, 7, -1, -1, -1, -1, -1))


def test_barycentric_known(oracle):
    # test_celltree.py:528-588
    t = oracle.OracleCellTree2d(NODES2, FACES2, -1)
    idx, w = t.compute_barycentric_weights(np.array([[0.0, 0.0], [1.0, 1.0], [2.0, 1.0]]))
    assert np.array_equal(idx, [0, 0, 1])
    assert np.allclose(w, [[1.0, 0.0, 0.0], [0.25, 0.25, 0.5], [0.5, 0.25, 0.25]])
    nodes = np.array([[0.0, 0.0], [2.0, 0.0], [2.0, 2.0], [0.0, 2.0], [4.0, 0.0], [4.0, 4.0]])
    t = oracle.OracleCellTree2d(nodes, np.array([[0, 1, 2, 3], [1, 4, 5, 2]]), -1)
    idx, w = t.compute_barycentric_weights(np.array([[0.0, 0.0], [1.0, 1.0], [2.0, 1.0]]))
    assert np.array_equal(idx, [0, 0, 0])
    assert np.allclose(w, [[1, 0, 0, 0], [0.25, 0.25, 0.25, 0.25], [0, 0.5, 0.5, 0]])


def test_edge_tree_known(oracle):
    # test_edgecelltree.py:12-92
    v = np.array([[0.0, 0.0], [1.0, 0.0], [2.0, 0.0], [2.0, 1.0]])
    e = np.array([[0, 1], [1, 2], [2, 3]], dtype=np.int32)
    t = oracle.OracleEdgeCellTree2d(v, e)
    assert t.nodes.shape == (3,)
    assert np.array_equal(t.bb_indices, [0, 1, 2])
    assert np.allclose(t.bb_coords, [[0, 1, 0, 0], [1, 2, 0, 0], [2, 2, 0, 1]], atol=1e-9)
    assert np.array_equal(t.locate_points(np.array([[0.5, 0.0], [1.5, 0.0], [2.0, 0.5]])), [0, 1, 2])
    assert np.array_equal(t.locate_points(np.array([[0.5, 0.5], [1.5, 0.5], [2.0, 0.5]])), [-1, -1, 2])
    vv = np.array([[171805.657000002, 563516.366], [171889.594000001, 563437.333000001]])
    t2 = oracle.OracleEdgeCellTree2d(vv, np.array([[0, 1]]))
    p = np.array([[171882.49385095935, 563444.0183244612]])
    assert np.array_equal(t2.locate_points(p, tolerance=1e-8), [0])
    assert np.array_equal(t2.locate_points(p, tolerance=1e-9), [0])
    segs = np.array([[[1.0, -1.0], [1.0, 1.0]], [[3.0, 1.0], [-1.0, -1.0]], [[0.0, -1.0], [0.0, 1.0]],
                     [[-2.0, -1.0], [-3.0, -1.0]]])
    i, j, xy = t.intersect_edges(segs)
    assert np.array_equal(i, [0, 1, 1]) and np.array_equal(j, [0, 2, 1])
    assert np.allclose(xy, [[1.0, 0.0], [2.0, 0.5], [1.0, 0.0]], atol=1e-9)


def test_tolerance_helpers(oracle):
    # test_celltree_utils.py:19-52
    assert np.isclose(oracle.default_tolerance(np.array([2.4, 0.5])), 2.4e-12, rtol=0, atol=1e-20)
    assert oracle.default_tolerance(np.array([2.4, 0.5]) / 1e4) == 1e-15
    bb = np.array([[1.0, 2.0, 1.0, 2.0], [4.0, 5.0, 0.0, 1.0], [4.0, 5.0, 2.0, 3.0], [-1.0, 0.0, 0.0, 4.0],
                   [6.0, 8.0, 0.0, 4.0], [0.0, 6.0, -1.0, 0.0], [0.0, 6.0, 4.0, 5.0]])
    assert np.allclose(oracle.bbox_tree(bb), [-1.0, 8.0, -1.0, 5.0])
    d = oracle.bbox_distances(bb)
    assert np.allclose(d[:, 2], [1.41421356, 1.41421356, 1.41421356, 4.12310563, 4.47213595, 6.08276253,
                                 6.08276253])


def test_counter_clockwise_and_sort(oracle):
    # test_geometry_utils.py:319-348 and 476-505
    v = np.array([[0.0, 0.0], [0.5, 0.0], [1.0, 0.0], [1.0, 0.5], [1.0, 1.0], [0.0, 1.0]])
    ccw = np.array([[0, 2, 4, 5, -1, -1], [0, 1, 2, 3, 4, 5]], dtype=np.int64)
    cw = np.array([[5, 4, 2, 0, -1, -1], [5, 4, 3, 2, 1, 0]], dtype=np.int64)
    e = ccw.copy()
    oracle.counter_clockwise(v, ccw)
    assert np.array_equal(ccw, e)
    oracle.counter_clockwise(v, cw)
    assert np.array_equal(cw, e)
