"""Density ingest from .pvti / .vti files (example_kitchensink.py:7-36's
pvti_readin, which needs vtk; vtk is not installed, so the files here are
written by hand in the VTK XML layout the VTK file-format documentation
gives: ImageData / PImageData, DataArrays in ascii, inline binary and
appended (raw and base64) form, UInt32 and UInt64 headers, zlib blocks).

The reference's reader returns the first cell-data array reshaped in Fortran
order over the cell counts, i.e. img[ix, iy, iz] is cell (ix, iy, iz) with x
fastest in the file; vector arrays get a trailing component axis."""
import base64
import os
import zlib

import numpy as np
import pytest

from tests.conftest import GOLDEN
from turbulence_tracing_gb300 import vtk_io


def _b64_runs(header, data):
    """VTK's inline/appended base64: header and data as separately padded runs."""
    return base64.b64encode(header) + base64.b64encode(data)


def _binary_blob(arr, header_t, compress, block=4096):
    raw = np.ascontiguousarray(arr).tobytes()
    if not compress:
        return np.array([len(raw)], header_t).tobytes(), raw
    blocks = [raw[i:i + block] for i in range(0, len(raw), block)] or [b""]
    comp = [zlib.compress(b) for b in blocks]
    last = len(blocks[-1]) if len(blocks[-1]) != block else block
    hdr = np.array([len(blocks), block, last] + [len(c) for c in comp], header_t).tobytes()
    return hdr, b"".join(comp)


def write_vti(path, cells, extent, spacing=(1.0, 1.0, 1.0), origin=(0.0, 0.0, 0.0), fmt="ascii",
              header="UInt32", compress=False, whole=None, extra_first=None):
    """cells: array (nz, ny, nx[, ncomp]) of the piece's cell values (x fastest in the file)."""
    header_t = np.uint64 if header == "UInt64" else np.uint32
    ncomp = cells.shape[3] if cells.ndim == 4 else 1
    flat = cells.reshape(-1, ncomp) if ncomp > 1 else cells.reshape(-1)
    tname = {np.float64: "Float64", np.float32: "Float32"}[cells.dtype.type]
    ext = " ".join(str(v) for v in extent)
    wext = " ".join(str(v) for v in (whole or extent))
    comp_attr = ' compressor="vtkZLibDataCompressor"' if compress else ""
    arrays = []
    if extra_first is not None:  # a point-data array first, which the reader must not take
        arrays.append(("PointData", "pts", extra_first))
    arrays.append(("CellData", "rnec", flat))
    body, appended = [], b""
    for where, name, a in arrays:
        nc = a.shape[1] if a.ndim == 2 else 1
        tn = {np.float64: "Float64", np.float32: "Float32"}[a.dtype.type]
        attrs = 'type="%s" Name="%s" NumberOfComponents="%d"' % (tn, name, nc)
        if fmt == "ascii":
            el = '<DataArray %s format="ascii">%s</DataArray>' % (attrs, " ".join(repr(float(v)) for v in a.ravel()))
        elif fmt == "binary":
            h, d = _binary_blob(a, header_t, compress)
            el = '<DataArray %s format="binary">%s</DataArray>' % (attrs, _b64_runs(h, d).decode())
        else:
            h, d = _binary_blob(a, header_t, compress)
            blob = (h + d) if fmt == "raw" else _b64_runs(h, d)
            el = '<DataArray %s format="appended" offset="%d"/>' % (attrs, len(appended))
            appended += blob
        body.append("<%s>%s</%s>" % (where, el, where))
    xml = ('<?xml version="1.0"?>\n<VTKFile type="ImageData" version="1.0" byte_order="LittleEndian" '
           'header_type="%s"%s>\n<ImageData WholeExtent="%s" Origin="%s" Spacing="%s">\n<Piece Extent="%s">\n%s\n'
           '</Piece>\n</ImageData>\n' % (header, comp_attr, wext, " ".join(map(str, origin)),
                                        " ".join(map(str, spacing)), ext, "\n".join(body)))
    out = xml.encode()
    if fmt in ("raw", "base64"):
        out += ('<AppendedData encoding="%s">\n   _' % ("raw" if fmt == "raw" else "base64")).encode()
        out += appended + b"\n</AppendedData>\n"
    out += b"</VTKFile>\n"
    with open(path, "wb") as f:
        f.write(out)


def write_pvti(path, cells, splits, spacing, **kw):
    """cells (nz, ny, nx[, c]); splits: cell boundaries along z for the pieces."""
    nz, ny, nx = cells.shape[:3]
    whole = (0, nx, 0, ny, 0, nz)
    base = os.path.splitext(os.path.basename(path))[0]
    pieces = []
    for i, (k0, k1) in enumerate(zip(splits[:-1], splits[1:])):
        src = "%s_%d.vti" % (base, i)
        ext = (0, nx, 0, ny, k0, k1)
        write_vti(os.path.join(os.path.dirname(path), src), cells[k0:k1], ext, spacing=spacing, whole=whole, **kw)
        pieces.append('<Piece Extent="%s" Source="%s"/>' % (" ".join(map(str, ext)), src))
    tn = {np.float64: "Float64", np.float32: "Float32"}[cells.dtype.type]
    nc = cells.shape[3] if cells.ndim == 4 else 1
    xml = ('<?xml version="1.0"?>\n<VTKFile type="PImageData" version="1.0" byte_order="LittleEndian">\n'
           '<PImageData WholeExtent="%s" GhostLevel="0" Origin="0 0 0" Spacing="%s">\n'
           '<PCellData Scalars="rnec"><PDataArray type="%s" Name="rnec" NumberOfComponents="%d"/></PCellData>\n'
           '%s\n</PImageData>\n</VTKFile>\n' % (" ".join(map(str, whole)), " ".join(map(str, spacing)), tn, nc,
                                                "\n".join(pieces)))
    with open(path, "w") as f:
        f.write(xml)


def _reference_layout(cells):
    """What the reference's reader returns for these cells: img[ix, iy, iz(, c)]."""
    return np.moveaxis(cells, (0, 1, 2), (2, 1, 0))


@pytest.mark.parametrize("fmt,header,compress", [("ascii", "UInt32", False), ("binary", "UInt32", False),
                                                 ("binary", "UInt64", True), ("raw", "UInt64", False),
                                                 ("raw", "UInt32", True), ("base64", "UInt32", False),
                                                 ("base64", "UInt64", True)])
def test_pvti_readin_formats(tmp_path, fmt, header, compress):
    rng = np.random.default_rng(3)
    cells = rng.random((7, 5, 6)) * 1e25  # (nz, ny, nx)
    path = str(tmp_path / "ne.pvti")
    write_pvti(path, cells, [0, 3, 7], (2e-5, 3e-5, 4e-5), fmt=fmt, header=header, compress=compress)
    img, dim, spacing = vtk_io.pvti_readin(path)
    assert dim == (6, 5, 7) and img.shape == dim
    assert np.array_equal(img, _reference_layout(cells))
    assert np.allclose(spacing, [2e-5, 3e-5, 4e-5])


def test_vector_cell_data_and_point_data_skipped(tmp_path):
    rng = np.random.default_rng(4)
    cells = rng.random((4, 3, 5, 3)).astype(np.float32)  # a 3-vector per cell (e.g. the B field)
    pts = rng.random(6 * 4 * 5)
    path = str(tmp_path / "b.vti")
    write_vti(path, cells, (0, 5, 0, 3, 0, 4), fmt="raw", compress=True, extra_first=pts)
    img, dim, _ = vtk_io.pvti_readin(path)
    assert dim == (5, 3, 4, 3)
    assert np.array_equal(img, _reference_layout(cells))


def test_committed_ascii_fixture():
    """A hand-written ascii .pvti with two .vti pieces (tests/golden/vtk/): the
    cell value encodes its index, 100 ix + 10 iy + iz."""
    img, dim, spacing = vtk_io.pvti_readin(os.path.join(GOLDEN, "vtk", "rnec.pvti"))
    assert dim == (3, 2, 4)
    ix, iy, iz = np.meshgrid(np.arange(3), np.arange(2), np.arange(4), indexing="ij")
    assert np.array_equal(img, 100.0 * ix + 10.0 * iy + iz)
    assert np.allclose(spacing, [1e-5, 1e-5, 2e-5])


def test_feeds_electron_cube(tmp_path):
    """The reader's output is an ElectronCube density as the kitchen-sink example uses it."""
    from turbulence_tracing_gb300 import particle_tracker as pt

    cells = np.full((4, 4, 4), 1e24)
    path = str(tmp_path / "c.pvti")
    write_pvti(path, cells, [0, 2, 4], (1e-5, 1e-5, 1e-5), fmt="raw")
    rnec, dim, spacing = vtk_io.pvti_readin(path)
    x = np.linspace(-1.5e-5, 1.5e-5, dim[0])
    cube = pt.ElectronCube(x, x, x)
    cube.external_ne(rnec)
    assert cube.ne.shape == (4, 4, 4)
