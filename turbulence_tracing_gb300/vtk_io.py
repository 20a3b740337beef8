"""Density ingest from VTK XML image files, without vtk.

Replaces ``pvti_readin`` of particle_tracking/example_kitchensink.py:7-36,
which reads a simulation's electron density (``.pvti``, the parallel image
format whose pieces are ``.vti`` files) through vtkXMLPImageDataReader and
returns the first cell-data array as a numpy array.  This module parses the
same files with the standard library and numpy: the VTK XML ImageData and
PImageData formats with DataArrays in ``ascii``, inline ``binary`` (base64)
or ``appended`` (raw or base64) form, a UInt32 or UInt64 block header, and
optional zlib compression (vtkZLibDataCompressor).

``pvti_readin(filename)`` returns ``(img, dim, spacing)`` exactly as the
reference does: ``img`` the first cell-data array over the whole extent,
indexed ``[ix, iy, iz]`` (``[ix, iy, iz, comp]`` for vector arrays), ``dim``
its shape and ``spacing`` the grid spacing.  The result feeds
``ElectronCube.external_ne`` directly.
"""
import base64
import os
import xml.etree.ElementTree as ET
import zlib

import numpy as np

_TYPES = {"Int8": np.int8, "UInt8": np.uint8, "Int16": np.int16, "UInt16": np.uint16, "Int32": np.int32,
          "UInt32": np.uint32, "Int64": np.int64, "UInt64": np.uint64, "Float32": np.float32,
          "Float64": np.float64}


class _File:
    """One parsed VTK XML file: its root element, byte order, header type,
    compressor and appended-data block."""

    def __init__(self, path):
        with open(path, "rb") as f:
            raw = f.read()
        # the appended block is raw bytes after an underscore; keep it out of the XML parser
        start = raw.find(b"<AppendedData")
        self.appended = None
        self.appended_encoding = None
        if start >= 0:
            tag_end = raw.index(b">", start)
            head = raw[start:tag_end + 1].decode("ascii", "replace")
            self.appended_encoding = "base64" if 'encoding="base64"' in head else "raw"
            us = raw.index(b"_", tag_end)
            stop = raw.rfind(b"</AppendedData>")
            body = raw[us + 1:stop]
            if self.appended_encoding == "base64":
                body = body.strip()
            self.appended = body  # raw bytes: each array's own header gives its length
            raw = raw[:start] + b"<AppendedData/>" + raw[stop + len(b"</AppendedData>"):]
        self.root = ET.fromstring(raw)
        if self.root.tag != "VTKFile":
            raise ValueError("%s: not a VTK XML file" % path)
        self.order = "<" if self.root.get("byte_order", "LittleEndian") == "LittleEndian" else ">"
        self.header = np.dtype(self.order + ("u8" if self.root.get("header_type", "UInt32") == "UInt64" else "u4"))
        self.compressed = self.root.get("compressor", "") != ""
        if self.compressed and "ZLib" not in self.root.get("compressor", ""):
            raise NotImplementedError("%s: compressor %s (only zlib is supported)" % (path, self.root.get("compressor")))

    def _blocks(self, buf):
        """Decode one header-prefixed (optionally zlib-compressed) binary array from bytes."""
        h = self.header.itemsize
        if not self.compressed:
            n = int(np.frombuffer(buf[:h], self.header)[0])
            return buf[h:h + n], h + n
        nb = int(np.frombuffer(buf[:h], self.header)[0])
        hdr = np.frombuffer(buf[:h * (3 + nb)], self.header)
        sizes = hdr[3:3 + nb].astype(np.int64)
        off = h * (3 + nb)
        parts = []
        for sz in sizes:
            parts.append(zlib.decompress(buf[off:off + int(sz)]))
            off += int(sz)
        return b"".join(parts), off

    def _blocks_b64(self, text):
        """Base64 (inline binary, or appended with encoding="base64"): VTK encodes
        the header and the data as two separately padded base64 runs; an
        uncompressed array written as one run is read too."""
        h = self.header.itemsize
        if isinstance(text, str):
            text = text.encode()
        if not self.compressed:
            henc = ((h + 2) // 3) * 4
            if h % 3 and text[henc - 1:henc] != b"=":  # header and data in one run
                head = base64.b64decode(text[:((h + 2) // 3 + 1) * 4])
                n = int(np.frombuffer(head[:h], self.header)[0])
                return base64.b64decode(text[:((h + n + 2) // 3) * 4])[h:h + n]
            n = int(np.frombuffer(base64.b64decode(text[:henc])[:h], self.header)[0])
            return base64.b64decode(text[henc:henc + ((n + 2) // 3) * 4])[:n]
        first = base64.b64decode(text[:((3 * h + 2) // 3) * 4])
        nb = int(np.frombuffer(first[:h], self.header)[0])
        hlen = h * (3 + nb)
        henc = ((hlen + 2) // 3) * 4
        hdr = base64.b64decode(text[:henc])[:hlen]
        sizes = np.frombuffer(hdr, self.header)[3:3 + nb].astype(np.int64)
        total = int(sizes.sum())
        data = base64.b64decode(text[henc:henc + ((total + 2) // 3) * 4])[:total]
        parts, off = [], 0
        for sz in sizes:
            parts.append(zlib.decompress(data[off:off + int(sz)]))
            off += int(sz)
        return b"".join(parts)

    def array(self, el):
        """numpy array of a <DataArray> element: (ntuples,) or (ntuples, ncomp)."""
        dt = np.dtype(self.order + np.dtype(_TYPES[el.get("type")]).str[1:])
        ncomp = int(el.get("NumberOfComponents", "1"))
        fmt = el.get("format", "ascii")
        if fmt == "ascii":
            a = np.array((el.text or "").split(), dtype=dt)
        elif fmt == "binary":
            a = np.frombuffer(self._blocks_b64("".join((el.text or "").split()).encode()), dtype=dt)
        elif fmt == "appended":
            off = int(el.get("offset", "0"))
            if self.appended is None:
                raise ValueError("DataArray is appended but the file has no AppendedData")
            if self.appended_encoding == "raw":
                a = np.frombuffer(self._blocks(self.appended[off:])[0], dtype=dt)
            else:
                a = np.frombuffer(self._blocks_b64(self.appended[off:]), dtype=dt)
        else:
            raise ValueError("DataArray format %r" % fmt)
        a = a.astype(dt.newbyteorder("="), copy=False)
        return a.reshape(-1, ncomp) if ncomp > 1 else a


def _extent(s):
    e = [int(v) for v in s.split()]
    if len(e) != 6:
        raise ValueError("extent needs 6 integers: %r" % s)
    return e


def _cell_array(vf, piece, name=None):
    cd = piece.find("CellData")
    arrays = [] if cd is None else cd.findall("DataArray")
    if not arrays:
        raise ValueError("piece has no cell data")
    el = arrays[0] if name is None else next(a for a in arrays if a.get("Name") == name)
    return el.get("Name"), vf.array(el)


def read_image_cells(filename, name=None):
    """First (or the named) cell-data array of a .vti or .pvti file over the whole
    extent, in VTK's x-fastest order: returns (flat array (ncells[, ncomp]),
    point dimensions (nx, ny, nz), spacing, origin)."""
    vf = _File(filename)
    kind = vf.root.get("type")
    if kind == "ImageData":
        img = vf.root.find("ImageData")
        whole = _extent(img.get("WholeExtent"))
        pieces = [(vf, p) for p in img.findall("Piece")]
    elif kind == "PImageData":
        img = vf.root.find("PImageData")
        whole = _extent(img.get("WholeExtent"))
        base = os.path.dirname(os.path.abspath(filename))
        pieces = []
        for p in img.findall("Piece"):
            sub = _File(os.path.join(base, p.get("Source")))
            sp = sub.root.find("ImageData").findall("Piece")
            if len(sp) != 1:
                raise ValueError("%s: expected one piece" % p.get("Source"))
            pieces.append((sub, sp[0]))
    else:
        raise ValueError("%s: VTK file type %r is not image data" % (filename, kind))
    spacing = np.array([float(v) for v in img.get("Spacing", "1 1 1").split()])
    origin = np.array([float(v) for v in img.get("Origin", "0 0 0").split()])
    dims = [whole[1] - whole[0] + 1, whole[3] - whole[2] + 1, whole[5] - whole[4] + 1]
    cells = [max(d - 1, 1) for d in dims]
    out = None
    for pf, piece in pieces:
        pe = _extent(piece.get("Extent"))
        nm, a = _cell_array(pf, piece, name)
        name = nm if name is None else name
        pc = [max(pe[1] - pe[0], 1), max(pe[3] - pe[2], 1), max(pe[5] - pe[4], 1)]
        ncomp = a.shape[1] if a.ndim == 2 else 1
        if a.shape[0] != pc[0] * pc[1] * pc[2]:
            raise ValueError("piece %s holds %d cells, its extent %d" % (piece.get("Extent"), a.shape[0],
                                                                          pc[0] * pc[1] * pc[2]))
        if out is None:
            out = np.empty((cells[2], cells[1], cells[0]) + ((ncomp,) if ncomp > 1 else ()), dtype=a.dtype)
        blk = a.reshape((pc[2], pc[1], pc[0]) + ((ncomp,) if ncomp > 1 else ()))
        i0, j0, k0 = pe[0] - whole[0], pe[2] - whole[2], pe[4] - whole[4]
        out[k0:k0 + pc[2], j0:j0 + pc[1], i0:i0 + pc[0]] = blk
    flat = out.reshape((cells[0] * cells[1] * cells[2],) + out.shape[3:])
    return flat, tuple(dims), spacing, origin


def pvti_readin(filename):
    """The reference's reader (example_kitchensink.py:7-36): the first cell-data
    array of a .pvti (or .vti) file as img[ix, iy, iz] (img[ix, iy, iz, comp] for
    vectors), its shape, and the grid spacing."""
    v, dim, spacing, _ = read_image_cells(filename)
    n_comp = v.shape[1] if v.ndim == 2 else 1
    vec = [int(i - 1) for i in dim]
    if n_comp > 1:
        vec.append(n_comp)
    if n_comp > 2:
        img = v.reshape(vec, order="F")[0:dim[0] - 1, 0:dim[1] - 1, 0:dim[2] - 1, :]
    else:
        img = v.reshape(vec, order="F")[0:dim[0] - 1, 0:dim[1] - 1, 0:dim[2] - 1]
    return img, img.shape, spacing
