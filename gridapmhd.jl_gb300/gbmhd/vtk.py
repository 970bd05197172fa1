"""VTK output of the solution fields, as hunt(..., vtk=true) writes them
(src/Applications/hunt.jl:263-273): an unstructured grid of order 2, each cell split into eight
linear hexahedra over its 27 Q2 nodes, with the fields at the nodes as point data (the nodes of
each cell are its own, so discontinuous fields stay discontinuous).  The fields are evaluated on
the device (gbmhd_node_fields); this module only writes the XML file (raw appended binary)."""
from __future__ import annotations

import numpy as np

FIELDS = (("uh", slice(3, 6)), ("ph", slice(6, 7)), ("jh", slice(7, 10)), ("phi", slice(10, 11)),
          ("div_uh", slice(11, 12)), ("div_jh", slice(12, 13)))
_VTK_HEXAHEDRON = 12


def sub_hexes() -> np.ndarray:
    """(8, 8) node ids (n = a + 3b + 9c) of the eight linear sub-hexahedra, VTK vertex order."""
    out = []
    for c in range(2):
        for b in range(2):
            for a in range(2):
                n = lambda i, j, k: (a + i) + 3 * (b + j) + 9 * (c + k)
                out.append([n(0, 0, 0), n(1, 0, 0), n(1, 1, 0), n(0, 1, 0),
                             n(0, 0, 1), n(1, 0, 1), n(1, 1, 1), n(0, 1, 1)])
    return np.array(out, np.int64)


def write_vtu(path: str, node_fields: np.ndarray) -> str:
    """Write node_fields (ncells, 27, 13) to path (.vtu appended) and return the path."""
    nf = np.ascontiguousarray(node_fields, np.float64)
    ncells = nf.shape[0]
    pts = nf[:, :, 0:3].reshape(-1, 3)
    conn = (sub_hexes()[None, :, :] + 27 * np.arange(ncells)[:, None, None]).reshape(-1)
    nsub = 8 * ncells
    offsets = 8 * np.arange(1, nsub + 1, dtype=np.int64)
    types = np.full(nsub, _VTK_HEXAHEDRON, np.uint8)
    arrays = [("Points", pts, 3)]
    for name, sl in FIELDS:
        a = nf[:, :, sl].reshape(-1, sl.stop - sl.start)
        arrays.append((name, a, sl.stop - sl.start))
    blobs, offset, xml_pd = [], 0, []

    def add(arr):
        nonlocal offset
        raw = np.ascontiguousarray(arr).tobytes()
        blob = np.uint64(len(raw)).tobytes() + raw
        blobs.append(blob)
        o = offset
        offset += len(blob)
        return o

    o_pts = add(pts)
    for name, a, nc in arrays[1:]:
        o = add(a)
        xml_pd.append(f'        <DataArray type="Float64" Name="{name}" NumberOfComponents="{nc}" format="appended" '
                      f'offset="{o}"/>')
    o_conn, o_off, o_typ = add(conn.astype(np.int64)), add(offsets), add(types)
    head = "\n".join([
        '<?xml version="1.0"?>',
        '<VTKFile type="UnstructuredGrid" version="1.0" byte_order="LittleEndian" header_type="UInt64">',
        '  <UnstructuredGrid>',
        f'    <Piece NumberOfPoints="{len(pts)}" NumberOfCells="{nsub}">',
        '      <PointData>', *xml_pd, '      </PointData>',
        '      <Points>',
        f'        <DataArray type="Float64" NumberOfComponents="3" format="appended" offset="{o_pts}"/>',
        '      </Points>',
        '      <Cells>',
        f'        <DataArray type="Int64" Name="connectivity" format="appended" offset="{o_conn}"/>',
        f'        <DataArray type="Int64" Name="offsets" format="appended" offset="{o_off}"/>',
        f'        <DataArray type="UInt8" Name="types" format="appended" offset="{o_typ}"/>',
        '      </Cells>',
        '    </Piece>',
        '  </UnstructuredGrid>',
        '  <AppendedData encoding="raw">',
        '_'])
    with open(path, "wb") as fh:
        fh.write(head.encode())
        for b in blobs:
            fh.write(b)
        fh.write(b"\n  </AppendedData>\n</VTKFile>\n")
    return path


def read_vtu_arrays(path: str) -> dict:
    """Read back the arrays of a file written by write_vtu (for tests)."""
    import re
    data = open(path, "rb").read()
    start = data.index(b"<AppendedData encoding=\"raw\">")
    us = data.index(b"_", start) + 1
    head = data[:start].decode()
    out = {}
    for m in re.finditer(r'<DataArray type="(\w+)"(?: Name="(\w+)")?(?: NumberOfComponents="(\d+)")? format="appended" '
                         r'offset="(\d+)"', head):
        typ, name, nc, off = m.group(1), m.group(2) or "Points", int(m.group(3) or 1), int(m.group(4))
        n = int(np.frombuffer(data[us + off:us + off + 8], np.uint64)[0])
        dt = {"Float64": np.float64, "Int64": np.int64, "UInt8": np.uint8}[typ]
        a = np.frombuffer(data[us + off + 8:us + off + 8 + n], dt)
        out[name] = a.reshape(-1, nc) if nc > 1 else a
    return out
