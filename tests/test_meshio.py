"""mesh-part's files and points: MEDIT ASCII meshes, "MeWe" weight files and
"MePe" partition files (coupe's mesh-io crate) on the host, and the element
barycentres on the GPU (tools/lib/lib.rs:511-539), then the whole
file-in, file-out flow.

CPU: byte layouts from mesh-io's encoders (weight.rs:123-191,
partition.rs:71-86), round trips, the parser's rules (parser.rs:189-380) and
its errors, the oracle's barycentres on hand-computed cases.  GPU: the
barycentre kernel against the oracle (bit-identical), its errors, and
mesh_part against the same steps done with the oracle.
"""
import struct

import numpy as np
import pytest

from coupe_gb300 import meshio

SMALL_3D = """MeshVersionFormatted 2
Dimension
3
Vertices
5
0 0 0 1
1 0 0 1
0 1 0 2
0 0 1 2
1 1 1 3
Corners 1
1
Tetrahedra 2
1 2 3 4 7
2 3 4 5 8
Triangles
1
1 2 3 5
END
"""


# ------------------------------------------------------------------ files
def test_partition_file_layout_and_round_trip(tmp_path):
    p = tmp_path / "p.mepe"
    meshio.write_partition(p, [3, 0, 2**40])
    data = p.read_bytes()
    assert data == b"MePe" + struct.pack("<Q", 3) + struct.pack("<3Q", 3, 0, 2**40)
    assert list(meshio.read_partition(p)) == [3, 0, 2**40]
    meshio.write_partition(p, [])
    assert p.read_bytes() == b"MePe" + bytes(8)
    assert len(meshio.read_partition(p)) == 0


def test_partition_file_errors(tmp_path):
    p = tmp_path / "p.mepe"
    p.write_bytes(b"MePx" + bytes(8))
    with pytest.raises(meshio.MeshIoError) as e:
        meshio.read_partition(p)
    assert e.value.kind == "bad_header"
    p.write_bytes(b"MePe" + struct.pack("<Q", 2) + bytes(8))  # one id short
    with pytest.raises(meshio.MeshIoError) as e:
        meshio.read_partition(p)
    assert e.value.kind == "io"


def test_weight_file_layout_and_round_trip(tmp_path):
    p = tmp_path / "w.mewe"
    meshio.write_weights(p, np.array([[5], [-7]], dtype=np.int64))
    assert p.read_bytes() == b"MeWe" + bytes([1, 1]) + struct.pack("<H", 1) + struct.pack("<Q", 2) + \
        struct.pack("<2q", 5, -7)
    kind, a = meshio.read_weights(p)
    assert kind == "integers" and a.dtype == np.int64 and a.tolist() == [[5], [-7]]
    meshio.write_weights(p, np.array([0.5, 2.25]))
    assert p.read_bytes()[4:8] == bytes([1, 0, 1, 0])
    kind, a = meshio.read_weights(p)
    assert kind == "floats" and a.tolist() == [[0.5], [2.25]]
    # empty: the 16-byte header with no criterion (weight.rs:148-156); read back as no integers
    meshio.write_weights(p, np.zeros((0, 1), dtype=np.int64))
    assert p.read_bytes() == b"MeWe" + bytes([1, 1, 0, 0]) + bytes(8)
    kind, a = meshio.read_weights(p)
    assert kind == "integers" and a.size == 0
    # coupe's writer asserts fewer than two criteria (weight.rs:159-162)
    with pytest.raises(ValueError):
        meshio.write_weights(p, np.ones((3, 2)))


def test_weight_file_reader_rules(tmp_path):
    p = tmp_path / "w.mewe"
    # several criteria are read (the reader has no limit), row by row
    p.write_bytes(b"MeWe" + bytes([1, 0]) + struct.pack("<H", 2) + struct.pack("<Q", 2) +
                  struct.pack("<4d", 1.0, 2.0, 3.0, 4.0))
    assert meshio.read_weights(p)[1].tolist() == [[1.0, 2.0], [3.0, 4.0]]
    p.write_bytes(b"MeWx" + bytes(12))
    with pytest.raises(meshio.MeshIoError) as e:
        meshio.read_weights(p)
    assert e.value.kind == "bad_header"
    p.write_bytes(b"MeWe" + bytes([2, 1, 1, 0]) + bytes(8))
    with pytest.raises(meshio.MeshIoError) as e:
        meshio.read_weights(p)
    assert e.value.kind == "unsupported_version"


# ------------------------------------------------------------ MEDIT ASCII
def test_medit_parse_small_mesh():
    m = meshio.parse_medit_ascii(SMALL_3D)
    assert m.dimension == 3
    assert m.coordinates.shape == (5, 3) and m.coordinates[4].tolist() == [1, 1, 1]
    assert m.node_refs.tolist() == [1, 1, 2, 2, 3]
    assert [t for t, _, _ in m.topology] == ["tetrahedron", "triangle"]
    tets = m.topology[0][1]
    assert tets.tolist() == [[0, 1, 2, 3], [1, 2, 3, 4]] and m.topology[0][2].tolist() == [7, 8]
    # the points are the tetrahedra's barycentres (largest dimension, edges never)
    blocks = meshio.element_blocks(m)
    assert [t for t, _ in blocks] == ["tetrahedron"]


def test_medit_parser_rules():
    # junk after an element keyword on its line is skipped; the count may follow
    txt = "MeshVersionFormatted 1 Dimension 2 Vertices 3\n0 0\n1 0\n0 1\nTriangles junk 1\n1 2 3\nEnd"
    m = meshio.parse_medit_ascii(txt)
    assert m.topology[0][1].tolist() == [[0, 1, 2]] and len(m.topology[0][2]) == 0
    # blank lines between entries are skipped; keywords in any case
    m = meshio.parse_medit_ascii("meshversionformatted 2\nDIMENSION 2\nvertices 1\n\n\n 3 4 9\nend\n")
    assert m.coordinates.tolist() == [[3, 4]] and m.node_refs.tolist() == [9]


@pytest.mark.parametrize("txt,kind", [
    ("MeshVersion 2", "unexpected_token"),
    ("MeshVersionFormatted 2 Dim 3", "unexpected_token"),
    ("MeshVersionFormatted 2 Dimension 2 Vertices 1\n0 0 1 5\nEnd", "unexpected_token"),
    ("MeshVersionFormatted 2 Dimension 2 Vertices 1\n0 x\nEnd", "bad_float"),
    ("MeshVersionFormatted 2 Dimension 2 Vertices 1\n0 0\nTriangles 1\n1 2\nEnd", "io"),
    ("MeshVersionFormatted 2 Dimension 2 Vertices 1\n0 0\nTriangles 1\n1 -2 3\nEnd", "bad_integer"),
    ("MeshVersionFormatted 2 Dimension 2 Vertices 1\n0 0\nTriangles\nx\n1\n1 2 3\nEnd", "bad_integer"),
    ("MeshVersionFormatted 2 Dimension 2 Vertices 1\n0 0\nPrisms 0\nEnd", "unexpected_token"),
    ("MeshVersionFormatted 2 Dimension 2 Vertices 1\n0 0\n", "io"),
])
def test_medit_parser_errors(txt, kind):
    with pytest.raises(meshio.MeshIoError) as e:
        meshio.parse_medit_ascii(txt)
    assert e.value.kind == kind


def test_medit_write_read_round_trip(tmp_path):
    m = meshio.parse_medit_ascii(SMALL_3D)
    p = tmp_path / "m.mesh"
    meshio.write_medit_ascii(p, m)
    m2 = meshio.read_medit(p)
    assert np.array_equal(m2.coordinates, m.coordinates)
    assert [(t, n.tolist(), r.tolist()) for t, n, r in m2.topology] == \
        [(t, n.tolist(), r.tolist()) for t, n, r in m.topology]


def test_oracle_barycentres_known_answers(oracle_mod):
    m = meshio.parse_medit_ascii(SMALL_3D)
    b = oracle_mod.barycentres(m.coordinates, m.topology[0][1])
    assert b.tolist() == [[0.25, 0.25, 0.25], [0.5, 0.5, 0.5]]


def _hex_mesh(nx, ny, nz, rng):
    """A structured hexahedral mesh with jittered nodes."""
    g = np.stack(np.meshgrid(np.arange(nx + 1), np.arange(ny + 1), np.arange(nz + 1), indexing="ij"), -1)
    coords = g.reshape(-1, 3).astype(np.float64) * (1.0, 10.0, 100.0) + rng.random(((nx + 1) * (ny + 1) * (nz + 1), 3))
    idx = np.arange(len(coords)).reshape(nx + 1, ny + 1, nz + 1)
    c = [idx[:-1, :-1, :-1], idx[1:, :-1, :-1], idx[1:, 1:, :-1], idx[:-1, 1:, :-1],
         idx[:-1, :-1, 1:], idx[1:, :-1, 1:], idx[1:, 1:, 1:], idx[:-1, 1:, 1:]]
    hexes = np.stack([a.reshape(-1) for a in c], -1).astype(np.uint64)
    return coords, hexes


# -------------------------------------------------------------------- GPU
@pytest.mark.gpu
def test_barycentres_match_oracle(coupe, oracle_mod):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(5)
    coords, hexes = _hex_mesh(40, 30, 20, rng)
    got = coupe.barycentres_host(coords, hexes)
    assert np.array_equal(got, oracle_mod.barycentres(coords, hexes))
    # triangles and quadrilaterals in 2D, tetrahedra in 3D, random node order
    for dim, k in ((2, 3), (2, 4), (3, 4), (3, 2)):
        c = rng.normal(size=(50_000, dim)) * 1e3
        nodes = rng.integers(0, len(c), (200_001, k)).astype(np.uint64)
        assert np.array_equal(coupe.barycentres_host(c, nodes), oracle_mod.barycentres(c, nodes)), (dim, k)
    # device tensors
    dc = torch.from_numpy(coords).cuda()
    dv = torch.from_numpy(hexes.astype(np.int64)).cuda()
    assert np.array_equal(coupe.barycentres_device(dc, dv).cpu().numpy(), oracle_mod.barycentres(coords, hexes))


@pytest.mark.gpu
def test_barycentre_errors(coupe):
    c = np.zeros((4, 3))
    with pytest.raises(coupe.CoupeError):
        coupe.barycentres_host(c, np.array([[0, 1, 2, 4]], dtype=np.uint64))  # node 4 of 4
    with pytest.raises(coupe.CoupeError):
        coupe.barycentres_host(c, np.array([[0, 1, 2, 3, 0]], dtype=np.uint64))  # 5 nodes
    with pytest.raises(coupe.CoupeError):
        coupe.barycentres_host(np.zeros((4, 4)), np.array([[0, 1, 2]], dtype=np.uint64))  # 4 coordinates
    # the context is still usable
    assert coupe.barycentres_host(c, np.array([[0, 1, 2, 3]], dtype=np.uint64)).tolist() == [[0, 0, 0]]


@pytest.mark.gpu
@pytest.mark.parametrize("algorithm", ["rcb", "rib"])
def test_mesh_part_file_flow(coupe, oracle_mod, tmp_path, algorithm):
    """mesh file + weight file -> partition file, against the same steps
    done with the oracle (barycentres, then Rcb / Rib on them)."""
    rng = np.random.default_rng(7)
    coords, hexes = _hex_mesh(30, 20, 12, rng)
    mesh = meshio.Mesh(dimension=3, coordinates=coords, node_refs=np.zeros(len(coords), dtype=np.int64),
                       topology=[("quadrilateral", hexes[:10, :4], np.zeros(0, dtype=np.int64)),
                                 ("hexahedron", hexes, np.zeros(0, dtype=np.int64))])
    meshio.write_medit_ascii(tmp_path / "m.mesh", mesh)
    w = rng.integers(1, 50, (len(hexes), 1)).astype(np.int64)
    meshio.write_weights(tmp_path / "w.mewe", w)
    ids = meshio.mesh_part(tmp_path / "m.mesh", tmp_path / "w.mewe", tmp_path / "p.mepe", algorithm=algorithm,
                           iter_count=5, tolerance=0.02)
    assert np.array_equal(meshio.read_partition(tmp_path / "p.mepe"), ids)
    pts = oracle_mod.barycentres(coords, hexes)  # quadrilaterals are not of the largest dimension
    if algorithm == "rcb":
        want, _ = oracle_mod.rcb(pts, w[:, 0], 5, 0.02)
    else:
        torch = pytest.importorskip("torch")
        M = coupe.rib_matrix_device(torch.from_numpy(pts).cuda())  # the basis change Rib applies
        want, _ = oracle_mod.rib(pts, w[:, 0], 5, 0.02, matrix=M)
    assert np.array_equal(ids, want)
