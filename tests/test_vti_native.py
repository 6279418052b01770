"""The library's VTI reader (dgx_vti_read_cells_size_origin / dgx_vti_read_dataset_int,
replacing f_VTI_readCellsSizeOrigin / f_VTI_readDataset_int of the reference,
src/grid/discretization_grid.h:19-22) through the C ABI, host only.

Known answers: the reference's 16x16x16 test geometry (TestVTI_readCellsSizeOrigin:
cells 16^3, size 1, origin 0; zlib blocks, Int64) and the 6-grain result geometry, read
the same as the Python reader; every encoding the reader accepts (ascii, raw and
zlib binary, UInt32 / UInt64 headers, several blocks, stored / fixed / dynamic deflate
blocks, integer types) round-trips; malformed content is refused with an error."""
import base64
import struct
import zlib

import numpy as np
import pytest

from solver_cpp_gb300 import DgxError, build, inputs, vti_read


@pytest.fixture(scope="module", autouse=True)
def _lib():
    build.build()


def _vti(cells, data, fmt="binary", header="UInt32", compress=None, dtype="<i8", block=None, name="material",
         origin=(0.5, -1.0, 2.0), spacing=(0.25, 0.5, 1.0)):
    vtype = {"<i1": "Int8", "<u1": "UInt8", "<i2": "Int16", "<u2": "UInt16", "<i4": "Int32", "<u4": "UInt32",
             "<i8": "Int64", "<u8": "UInt64"}[dtype]
    raw = np.asarray(data, dtype=dtype).tobytes()
    hfmt = "<I" if header == "UInt32" else "<Q"
    if fmt == "ascii":
        body = " ".join(str(int(x)) for x in data)
    elif compress is None:
        body = base64.b64encode(struct.pack(hfmt, len(raw))).decode() + base64.b64encode(raw).decode()
    else:
        bs = block or max(1, len(raw))
        chunks = [raw[k:k + bs] for k in range(0, len(raw), bs)] or [b""]
        comp = [compress(c) for c in chunks]
        hdr = struct.pack(hfmt, len(chunks)) + struct.pack(hfmt, bs) + struct.pack(hfmt, len(chunks[-1]))
        hdr += b"".join(struct.pack(hfmt, len(c)) for c in comp)
        body = base64.b64encode(hdr).decode() + base64.b64encode(b"".join(comp)).decode()
    comp_attr = ' compressor="vtkZLibDataCompressor"' if compress is not None else ""
    ext = " ".join(f"0 {c}" for c in cells)
    return (f'<?xml version="1.0"?>\n<VTKFile type="ImageData" version="1.0" byte_order="LittleEndian" '
            f'header_type="{header}"{comp_attr}>\n  <ImageData WholeExtent="{ext}" '
            f'Origin="{origin[0]} {origin[1]} {origin[2]}" Spacing="{spacing[0]} {spacing[1]} {spacing[2]}" '
            f'Direction="1 0 0 0 1 0 0 0 1">\n  <Piece Extent="{ext}">\n    <PointData/>\n    <CellData>\n'
            f'      <DataArray type="{vtype}" Name="{name}" format="{fmt}" RangeMin="0" RangeMax="1">\n'
            f'        {body}\n      </DataArray>\n    </CellData>\n  </Piece>\n  </ImageData>\n</VTKFile>\n')


def test_reference_16cube_known_answer(knowns):
    text = knowns["vti_16x16x16"]["content"]
    cells, size, origin, data = vti_read(text)
    assert list(cells) == [16, 16, 16] and list(size) == [1.0, 1.0, 1.0] and list(origin) == [0.0, 0.0, 0.0]
    c2, s2, o2, d2 = inputs.read_vti(text)
    assert np.array_equal(data, d2.astype(np.int32)) and data.size == 4096
    assert data.min() >= 0 and data.max() == 19


def test_reference_6grains_geometry(knowns):
    text = knowns["vti_6grains"]
    cells, size, origin, data = vti_read(text)
    c2, s2, o2, d2 = inputs.read_vti(text)
    assert list(cells) == list(c2) == [6, 7, 8]
    assert np.allclose(size, s2, rtol=0, atol=0) and np.allclose(origin, o2, rtol=0, atol=0)
    assert np.array_equal(data, d2.astype(np.int32))


@pytest.mark.parametrize("case", [
    dict(fmt="ascii", dtype="<i4"),
    dict(header="UInt32", dtype="<i8"),
    dict(header="UInt64", dtype="<i8"),
    dict(header="UInt64", dtype="<u2"),
    dict(compress=lambda b: zlib.compress(b, 6), dtype="<i8"),
    dict(compress=lambda b: zlib.compress(b, 0), dtype="<i4"),           # stored deflate blocks
    dict(compress=lambda b: zlib.compress(b, 1), dtype="<i1", block=50),  # several zlib blocks
    dict(compress=lambda b: zlib.compress(b, 9), header="UInt64", dtype="<u1", block=64),
])
def test_encodings_round_trip(case):
    rng = np.random.default_rng(5)
    cells = (7, 5, 3)
    data = rng.integers(0, 100, size=int(np.prod(cells)))
    text = _vti(cells, data, **case)
    c, s, o, d = vti_read(text)
    assert list(c) == list(cells)
    assert np.allclose(s, [7 * 0.25, 5 * 0.5, 3 * 1.0]) and list(o) == [0.5, -1.0, 2.0]
    assert np.array_equal(d, data.astype(np.int32))
    c2, s2, o2, d2 = inputs.read_vti(text)
    assert np.array_equal(d, d2.astype(np.int32))


def test_large_dynamic_huffman_blocks():
    # a 32^3 Voronoi map compresses with dynamic Huffman codes and long back references
    from solver_cpp_gb300.synthetic import voronoi
    cells = (32, 32, 32)
    data = voronoi(cells, (1, 1, 1), 40, 9)
    text = _vti(cells, data, compress=lambda b: zlib.compress(b, 6), block=32768)
    assert np.array_equal(vti_read(text)[3], data)


def test_malformed_content_is_refused():
    cells = (3, 2, 2)
    data = np.arange(12)
    good = _vti(cells, data, compress=lambda b: zlib.compress(b, 6))
    with pytest.raises(DgxError):
        vti_read(good, label="nonexistent")
    with pytest.raises(DgxError):
        vti_read(good.replace('type="ImageData"', 'type="PolyData"'))
    with pytest.raises(DgxError):
        vti_read(_vti(cells, data[:-1], fmt="ascii", dtype="<i4"))          # too few values
    # corrupt a compressed byte: the Adler-32 check or the decoder refuses it
    lines = good.split("\n")
    body = lines[[k for k, x in enumerate(lines) if "<DataArray" in x][0] + 1].strip()
    raw = bytearray(base64.b64decode(body[24:]))
    raw[len(raw) // 2] ^= 0x55
    bad = good.replace(body, body[:24] + base64.b64encode(bytes(raw)).decode())
    with pytest.raises(DgxError):
        vti_read(bad)
    with pytest.raises(DgxError):
        vti_read(_vti(cells, [0] * 11 + [2 ** 40], dtype="<i8"))              # beyond int32
