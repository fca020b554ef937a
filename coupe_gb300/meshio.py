"""Files of coupe's mesh tools, and the mesh-part flow around Rcb / Rib.

Host-side I/O, as in coupe's mesh-io crate:
  - MEDIT ASCII meshes (mesh-io/src/medit/parser.rs:189-380, `parse_ascii`),
  - weight files "MeWe" (mesh-io/src/weight.rs),
  - partition files "MePe" (mesh-io/src/partition.rs).
The points mesh-part partitions are the element barycentres
(tools/lib/lib.rs:511-539), computed on the GPU by coupe_gpu_barycentres;
`mesh_part` is mesh-part's file-in, file-out path (tools/bins/mesh-part.rs)
for Rcb and Rib.
"""
import struct
from dataclasses import dataclass, field

import numpy as np

# MEDIT section keyword -> (element type, dimension, node count)
# (mesh-io/src/lib.rs:25-54, medit/parser.rs:83-97)
ELEMENT_TYPES = {
    "edges": ("edge", 1, 2),
    "triangles": ("triangle", 2, 3),
    "quadrilaterals": ("quadrilateral", 2, 4),
    "quadrangles": ("quadrangle", 2, 4),
    "tetrahedra": ("tetrahedron", 3, 4),
    "hexahedra": ("hexahedron", 3, 8),
}
TYPE_DIM = {t: d for t, d, _ in ELEMENT_TYPES.values()}
TYPE_NODES = {t: k for t, _, k in ELEMENT_TYPES.values()}

WEIGHT_VERSION = 1
WEIGHT_FLAG_INTEGER = 1


class MeshIoError(Exception):
    """kind: "bad_header", "unsupported_version", "unexpected_token",
    "bad_integer", "bad_float" or "io" (mesh-io's error kinds)."""

    def __init__(self, kind, message, lineno=0):
        self.kind = kind
        self.lineno = lineno
        super().__init__("at line %d: %s" % (lineno, message) if lineno else message)


@dataclass
class Mesh:
    dimension: int = 0
    coordinates: np.ndarray = field(default_factory=lambda: np.zeros((0, 0)))  # (n_nodes, dimension)
    node_refs: np.ndarray = field(default_factory=lambda: np.zeros(0, dtype=np.int64))
    # [(element type, node lists (n_el, k) uint64 0-based, refs int64)], file order
    topology: list = field(default_factory=list)


# ---------------------------------------------------------------- MEDIT ASCII
class _Reader:
    """Tokens and lines as parse_ascii reads them: separators are space, tab,
    CR and LF; a line read first skips separators, then takes the rest of
    the line."""

    SEP = " \t\r\n"

    def __init__(self, text):
        self.t = text
        self.i = 0
        self.lineno = 1

    def _skip(self):
        t, i, n = self.t, self.i, len(self.t)
        while i < n and t[i] in self.SEP:
            if t[i] == "\n":
                self.lineno += 1
            i += 1
        if i >= n:
            raise MeshIoError("io", "unexpected end of file", self.lineno)
        self.i = i

    def token(self):
        self._skip()
        t, i, n = self.t, self.i, len(self.t)
        j = i
        while j < n and t[j] not in self.SEP:
            j += 1
        self.i = j
        return t[i:j].lower()

    def line(self):
        self._skip()
        j = self.t.find("\n", self.i)
        j = len(self.t) if j < 0 else j + 1
        s = self.t[self.i:j]
        self.i = j
        self.lineno += 1
        return s

    def lines(self, count):
        """`count` lines, each after skipping separators (blank lines)."""
        out = []
        for _ in range(count):
            out.append(self.line())
        return out


def _int(word, lineno, signed=False):
    """Rust's usize (or isize) parse: an optional sign ('-' only when
    signed), then decimal digits."""
    body = word[1:] if word[:1] in "+-" else word
    if not body.isdigit() or not body.isascii() or (word[:1] == "-" and not signed):
        raise MeshIoError("bad_integer", "when parsing integer: %r" % word, lineno)
    v = int(word, 10)
    if not (-(2**63) <= v < 2**63 if signed else v < 2**64):
        raise MeshIoError("bad_integer", "when parsing integer: %r (out of range)" % word, lineno)
    return v


def _float(word, lineno):
    try:
        if "_" in word or not word.isascii():
            raise ValueError
        return float(word)
    except ValueError:
        raise MeshIoError("bad_float", "when parsing float: %r" % word, lineno)


def parse_medit_ascii(text):
    """A Mesh from MEDIT ASCII text, as parse_ascii reads it: keywords are
    case-insensitive; Vertices lines hold `dimension` coordinates and an
    optional reference (anything more is an error); element lines hold the
    1-based node indices and an optional reference (words after it are
    ignored); Corners, Ridges and RequiredVertices are skipped; End ends the
    mesh; any other section is an error."""
    r = _Reader(text)
    tok = r.token()
    if tok != "meshversionformatted":
        raise MeshIoError("unexpected_token", "expected token 'MeshVersionFormatted', found %r" % tok, r.lineno)
    _int(r.token(), r.lineno)
    tok = r.token()
    if tok != "dimension":
        raise MeshIoError("unexpected_token", "expected token 'Dimension', found %r" % tok, r.lineno)
    dim = _int(r.token(), r.lineno)
    mesh = Mesh(dimension=dim, coordinates=np.zeros((0, dim)))
    while True:
        sec = r.token()
        if sec == "end":
            break
        if sec == "vertices":
            count = _int(r.token(), r.lineno)
            coords = np.zeros((count, dim))
            refs = []
            for v in range(count):
                words = r.line().split()
                if len(words) < dim:
                    raise MeshIoError("io", "unexpected end of line", r.lineno)
                for d in range(dim):
                    coords[v, d] = _float(words[d], r.lineno)
                if len(words) > dim:
                    refs.append(_int(words[dim], r.lineno, signed=True))
                if len(words) > dim + 1:
                    raise MeshIoError("unexpected_token", "expected token 'newline', found %r" % words[dim + 1],
                                      r.lineno)
            mesh.coordinates = coords
            mesh.node_refs = np.asarray(refs, dtype=np.int64)
        elif sec in ELEMENT_TYPES:
            etype, _, k = ELEMENT_TYPES[sec]
            first = r.lineno
            while True:  # junk on the keyword's line is skipped (parser.rs:288-304)
                word = r.token()
                try:
                    count = _int(word, r.lineno)
                    break
                except MeshIoError:
                    if r.lineno != first:
                        raise MeshIoError("bad_integer", "when parsing integer: %r" % word, first)
            nodes = np.zeros((count, k), dtype=np.uint64)
            refs = []
            for e in range(count):
                words = r.line().split()
                if len(words) < k:
                    raise MeshIoError("io", "unexpected end of line", r.lineno)
                for j in range(k):
                    v = _int(words[j], r.lineno)
                    if v == 0:
                        # usize `col - 1` underflows in coupe (a panic in debug builds)
                        raise MeshIoError("bad_integer", "node index 0 (indices start at 1)", r.lineno)
                    nodes[e, j] = v - 1
                if len(words) > k:
                    refs.append(_int(words[k], r.lineno, signed=True))
            mesh.topology.append((etype, nodes, np.asarray(refs, dtype=np.int64)))
        elif sec in ("corners", "ridges", "requiredvertices"):
            count = _int(r.token(), r.lineno)
            r.lines(count)
        else:
            raise MeshIoError("unexpected_token", "expected token 'element', found %r" % sec, r.lineno)
    return mesh


def read_medit(path):
    """A MEDIT ASCII mesh file (binary MEDIT files are not read here)."""
    with open(path, "rb") as f:
        data = f.read()
    if len(data) >= 4 and data[:4] in (b"\x01\x00\x00\x00", b"\x00\x00\x00\x01"):
        raise MeshIoError("unexpected_token", "binary MEDIT files are not supported; convert to ASCII")
    try:
        text = data.decode("utf-8")
    except UnicodeDecodeError as e:
        raise MeshIoError("io", str(e))
    return parse_medit_ascii(text)


def write_medit_ascii(path, mesh):
    """Writes a Mesh as MEDIT ASCII (1-based node indices; references
    written when present)."""
    with open(path, "w") as f:
        f.write("MeshVersionFormatted 2\nDimension %d\n" % mesh.dimension)
        n = len(mesh.coordinates)
        f.write("Vertices\n%d\n" % n)
        refs = mesh.node_refs if len(mesh.node_refs) == n else np.zeros(n, dtype=np.int64)
        for p, ref in zip(mesh.coordinates, refs):
            f.write(" ".join(repr(float(c)) for c in p) + " %d\n" % ref)
        names = {t: kw for kw, (t, _, _) in ELEMENT_TYPES.items()}
        for etype, nodes, erefs in mesh.topology:
            f.write("%s\n%d\n" % (names[etype].capitalize(), len(nodes)))
            er = erefs if len(erefs) == len(nodes) else np.zeros(len(nodes), dtype=np.int64)
            for row, ref in zip(nodes, er):
                f.write(" ".join(str(int(v) + 1) for v in row) + " %d\n" % ref)
        f.write("End\n")


# -------------------------------------------------------------- weight files
def read_weights(path):
    """A weight file (mesh-io/src/weight.rs:87-121): returns (kind, array)
    with kind "integers" (int64) or "floats" (float64) and array of shape
    (count, criteria).  No criterion: ("integers", empty) without reading
    further, as coupe does."""
    with open(path, "rb") as f:
        data = f.read()
    if len(data) < 4 or data[:4] != b"MeWe":
        raise MeshIoError("bad_header", "bad file header")
    if len(data) < 8:
        raise MeshIoError("io", "read/write error")
    version, flags, crit = data[4], data[5], struct.unpack_from("<H", data, 6)[0]
    if version != WEIGHT_VERSION:
        raise MeshIoError("unsupported_version", "unsupported file version")
    if crit == 0:
        return "integers", np.zeros((0, 0), dtype=np.int64)
    if len(data) < 16:
        raise MeshIoError("io", "read/write error")
    count = struct.unpack_from("<Q", data, 8)[0]
    need = 16 + count * crit * 8
    if len(data) < need:
        raise MeshIoError("io", "read/write error")
    dt = "<i8" if flags & WEIGHT_FLAG_INTEGER else "<f8"
    arr = np.frombuffer(data, dtype=dt, count=count * crit, offset=16).reshape(count, crit)
    kind = "integers" if flags & WEIGHT_FLAG_INTEGER else "floats"
    return kind, arr.astype(np.int64 if kind == "integers" else np.float64)


def write_weights(path, array):
    """A weight file (mesh-io/src/weight.rs:123-191): `array` of shape
    (count, criteria), int64 (integers) or float64 (floats).  Like coupe's
    writer, one criterion at most (its assertion rejects more); an empty
    array writes the 16-byte header with no criterion and count 0."""
    a = np.asarray(array)
    if a.ndim == 1:
        a = a.reshape(-1, 1)
    integer = a.dtype.kind in "iu"
    flags = WEIGHT_FLAG_INTEGER if integer else 0
    with open(path, "wb") as f:
        if len(a) == 0:
            f.write(b"MeWe" + bytes([WEIGHT_VERSION, flags, 0, 0]) + bytes(8))
            return
        crit = a.shape[1]
        if not crit < 2:
            raise ValueError("Too many criterions")
        f.write(b"MeWe" + bytes([WEIGHT_VERSION, flags]) + struct.pack("<H", crit) + struct.pack("<Q", len(a)))
        f.write(np.ascontiguousarray(a, dtype="<i8" if integer else "<f8").tobytes())


# ----------------------------------------------------------- partition files
def read_partition(path):
    """A partition file (mesh-io/src/partition.rs:45-69): uint64 part ids."""
    with open(path, "rb") as f:
        data = f.read()
    if len(data) < 4 or data[:4] != b"MePe":
        raise MeshIoError("bad_header", "bad file header")
    if len(data) < 12:
        raise MeshIoError("io", "read/write error")
    count = struct.unpack_from("<Q", data, 4)[0]
    if len(data) < 12 + 8 * count:
        raise MeshIoError("io", "read/write error")
    return np.frombuffer(data, dtype="<u8", count=count, offset=12).astype(np.uint64)


def write_partition(path, ids):
    """A partition file (mesh-io/src/partition.rs:71-86)."""
    a = np.ascontiguousarray(np.asarray(ids), dtype="<u8")
    with open(path, "wb") as f:
        f.write(b"MePe" + struct.pack("<Q", len(a)))
        f.write(a.tobytes())


# --------------------------------------------------------- mesh-part's flow
def element_blocks(mesh):
    """The element blocks whose barycentres are mesh-part's points
    (tools/lib/lib.rs:511-539): those of the largest element dimension,
    edges excepted, in file order."""
    if not mesh.topology:
        return []
    dim = max(TYPE_DIM[t] for t, _, _ in mesh.topology)
    return [(t, nodes) for t, nodes, _ in mesh.topology if TYPE_DIM[t] == dim and t != "edge"]


def barycentres(mesh):
    """mesh-part's points: the barycentres of element_blocks(mesh), computed
    on the GPU, as an (n, dimension) float64 array."""
    import coupe_gb300 as coupe
    blocks = element_blocks(mesh)
    if not blocks:
        return np.zeros((0, mesh.dimension))
    return np.concatenate([coupe.barycentres_host(mesh.coordinates, nodes) for _, nodes in blocks], axis=0)


def mesh_part(mesh_path, weights_path, out_path, algorithm="rcb", iter_count=1, tolerance=0.05, mode="ref32"):
    """mesh-part with one Rcb or Rib: reads the mesh and the weight file,
    partitions the element barycentres with the first weight criterion
    (tools/lib/lib.rs:212-229) and writes the partition file.  Returns the
    part ids."""
    import coupe_gb300 as coupe
    mesh = read_medit(mesh_path)
    kind, w = read_weights(weights_path)
    points = barycentres(mesh)
    weights = w[:, 0] if w.size else w.reshape(-1)
    ids = np.zeros(len(points), dtype=np.uint64)
    cls = {"rcb": coupe.Rcb, "rib": coupe.Rib}[algorithm]
    cls(iter_count=iter_count, tolerance=tolerance, mode=mode).partition(ids, (points, weights))
    write_partition(out_path, ids)
    return ids
