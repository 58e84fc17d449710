"""Host-side file contracts and the C ABI surface (no GPU needed).

Covers: every function declared in include/tdm.h is exported by libtdm.so;
extract_val semantics of the reference's KEY value files; the derived
geometry against the oracle; PGM reading (8/16-bit, comments, ROI); the
float32 multi-page TIFF writer.
"""
from __future__ import annotations

import ctypes

import os
import re
import struct

import numpy as np
import pytest

import oracle
from mtd_transmission_gb300 import api
from tests import simul
from mtd_transmission_gb300.api import Geometry
from tests.helpers import oracle_cfg

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _header_functions():
    txt = open(os.path.join(ROOT, "include", "tdm.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(tdm_\w+)\s*\(", txt)))


def test_library_exports_every_declared_function():
    lib = api.lib()
    declared = _header_functions()
    assert len(declared) >= 20
    missing = [f for f in declared if not hasattr(lib, f)]
    assert not missing, missing
    assert sorted(api.EXPORTS) == declared


def test_extract_val_semantics(tmp_path):
    f = tmp_path / "recon.txt"
    f.write_text("# comment\nNXMAX 64\n\n#NXMAX 99\nNA 1.40\nNA 1.2\nLAMBDA 0.000000633\nFLAG\nWIN 5\r\n")
    p = str(f)
    assert api.extract_val(p, "NXMAX") == (64.0, True)
    assert api.extract_val(p, "NA")[0] == float(np.float32(1.2))        # last occurrence wins, float-rounded
    assert api.extract_val(p, "LAMBDA")[0] == float(np.float32(6.33e-7))
    assert api.extract_val(p, "MISSING", 7.5) == (7.5, False)
    assert api.extract_val(p, "WIN")[0] == 5.0                           # trailing CR ignored by atof
    assert api.extract_val(p, "FLAG")[0] == 0.0                          # key without value reads 0
    assert api.extract_string(p, "NXMAX") == "64"
    with pytest.raises(api.TdmError):
        api.extract_val(str(tmp_path / "absent.txt"), "NXMAX")


@pytest.mark.parametrize("name", ["plain_512_born", "rytov_1024", "large_2048"])
def test_read_geom_and_derive(tmp_path, name):
    acq, _, _ = simul.workload(name)
    (tmp_path / "recon.txt").write_text(acq.recon_txt())
    (tmp_path / "config_manip.txt").write_text(acq.config_manip_txt())
    g = api.read_geom(str(tmp_path / "recon.txt"), str(tmp_path / "config_manip.txt"))
    ref = Geometry.from_acquisition(acq)
    for fname, _ in Geometry._fields_:
        assert getattr(g, fname) == getattr(ref, fname), fname
    d = api.derive(g)
    o = oracle.derive(oracle_cfg(acq))
    for k in ("rayon", "tp_holo", "tp_uborn", "tp_tomo", "delta_f"):
        assert d[k] == o[k], k


def _write_pgm(path, img, maxval, comment=True):
    h, w = img.shape
    hdr = b"P5\n" + (b"# written by the test\n" if comment else b"") + f"{w} {h}\n{maxval}\n".encode()
    data = img.astype(">u2").tobytes() if maxval > 255 else img.astype(np.uint8).tobytes()
    path.write_bytes(hdr + data)


def test_pgm_16bit_big_endian_roi(tmp_path):
    rng = np.random.default_rng(0)
    img = rng.integers(0, 4096, (40, 48), dtype=np.uint16)
    p = tmp_path / "i000.pgm"
    _write_pgm(p, img, 4095)
    out = api.read_pgm(str(p), 32)
    assert out.dtype == np.uint16
    np.testing.assert_array_equal(out, img[:32, :32])


def test_pgm_8bit(tmp_path):
    img = (np.arange(64 * 64) % 251).astype(np.uint8).reshape(64, 64)
    p = tmp_path / "mask.pgm"
    _write_pgm(p, img, 255, comment=False)
    out = api.read_pgm(str(p), 64)
    assert out.dtype == np.uint8
    np.testing.assert_array_equal(out, img)


def test_pgm_errors(tmp_path):
    img = np.zeros((16, 16), np.uint16)
    p = tmp_path / "t.pgm"
    _write_pgm(p, img, 4095)
    p.write_bytes(p.read_bytes()[:-10])          # truncated data
    with pytest.raises(api.TdmError):
        api.read_pgm(str(p), 16)
    with pytest.raises(api.TdmError):             # ROI larger than the image
        _write_pgm(p, img, 4095)
        api.read_pgm(str(p), 32)
    (tmp_path / "bad.pgm").write_bytes(b"P6\n2 2\n255\n" + bytes(12))
    with pytest.raises(api.TdmError):
        api.read_pgm(str(tmp_path / "bad.pgm"), 2)


def _read_tiff(path):
    """Minimal classic-TIFF reader: returns a list of (tags, float32 page)."""
    b = open(path, "rb").read()
    assert b[:4] == b"II*\x00"
    off = struct.unpack_from("<I", b, 4)[0]
    pages = []
    while off:
        n = struct.unpack_from("<H", b, off)[0]
        tags = {}
        for i in range(n):
            tag, typ, cnt, val = struct.unpack_from("<HHII", b, off + 2 + 12 * i)
            if typ == 3 and cnt == 1:
                val &= 0xFFFF
            if typ == 5:
                num, den = struct.unpack_from("<II", b, val)
                val = num / den
            tags[tag] = (val if not (typ == 3 and cnt == 2) else (val & 0xFFFF, val >> 16))
        w, h = tags[256], tags[257]
        data = np.frombuffer(b, "<f4", w * h, tags[273]).reshape(h, w)
        pages.append((tags, data))
        off = struct.unpack_from("<I", b, off + 2 + 12 * n)[0]
    return pages


def test_tiff_volume_roundtrip(tmp_path):
    rng = np.random.default_rng(2)
    vol = rng.standard_normal((5, 12, 16)).astype(np.float32)
    p = str(tmp_path / "indice.tif")
    api.write_tiff(p, vol, 1.1e-7)
    pages = _read_tiff(p)
    assert len(pages) == 5
    for z, (tags, data) in enumerate(pages):
        np.testing.assert_array_equal(data, vol[z])
        assert tags[258] == 32 and tags[339] == 3 and tags[274] == 4 and tags[296] == 3
        assert tags[285] == (z, 5)
        assert abs(tags[282] - 0.01 / np.float32(1.1e-7)) / tags[282] < 1e-6


def test_tiff_2d_topleft(tmp_path):
    img = np.arange(64, dtype=np.float32).reshape(8, 8)
    p = str(tmp_path / "centres.tif")
    api.write_tiff(p, img, 0.02, orientation=1)
    (tags, data), = _read_tiff(p)
    np.testing.assert_array_equal(data, img)
    assert tags[274] == 1


def test_no_cpu_fallback_without_a_gpu():
    """Without a CUDA device the library refuses the work (a status, an
    exception) instead of computing anything on the host."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present")
    acq, _, _ = simul.workload("plain_512_born")
    g = Geometry.from_acquisition(acq)
    with pytest.raises(api.TdmError):
        api.Context(g, 4)
    holos = np.zeros((2, acq.ccd_roix, acq.ccd_roix), np.uint16)
    out = np.full((2, 2 * acq.nxmax, 2 * acq.nxmax), np.nan, np.complex64)
    # host buffers: the C ABI itself refuses them (the Python wrapper refuses before the call)
    assert api.lib().tdm_extract_noalloc(ctypes.byref(g), api.ptr(holos), 16, 2, api.ptr(out), None) < api.TDM_OK
    assert np.isnan(out).all()  # nothing was written
    with pytest.raises(ValueError):
        api.extract_noalloc(g, holos, out, 0)


def test_noalloc_wrapper_checks_buffers():
    """The Python wrapper of the allocation-free extraction checks what the C
    ABI cannot see (buffer sizes, dtypes, devices) before calling it."""
    import torch
    acq, _, _ = simul.workload("plain_512_born")
    g = Geometry.from_acquisition(acq)
    H, F = acq.ccd_roix, 2 * acq.nxmax
    holos = torch.zeros((2, H, H), dtype=torch.uint16)
    out = torch.zeros((2, F, F), dtype=torch.complex64)
    with pytest.raises(ValueError, match="CUDA"):
        api.extract_noalloc(g, holos, out)
    with pytest.raises(ValueError):
        api.extract_noalloc(g, np.zeros((2, H, H), np.uint16), out)


def test_gather_angle_limit_refused_at_create():
    """The cap gather keeps each CTA's list of angles in shared memory: a
    context whose angle count cannot fit is refused at creation (before any
    device work), with the limit printed on stderr, instead of failing later."""
    acq, _, _ = simul.workload("rytov_1024")
    g = Geometry.from_acquisition(acq)
    with pytest.raises(api.TdmError) as e:
        api.Context(g, 40000)
    assert e.value.status == api.STATUS_CODES["TDM_EUNSUPPORTED"]


def test_reference_configuration_geometry():
    """tdm_read_geom on the reference's own Tomo_config gives the committed
    geometry (tests/golden/tomo_config_geometry.json), and the
    tomo_config_1024 workload is that geometry."""
    import json
    golden_path = os.path.join(os.path.dirname(__file__), "golden", "tomo_config_geometry.json")
    with open(golden_path) as f:
        golden = json.load(f)
    root = "/root/reference"
    if os.path.isdir(os.path.join(root, "Tomo_config")):
        sys_path = os.path.join(os.path.dirname(__file__), "golden")
        import importlib.util
        spec = importlib.util.spec_from_file_location("mk", os.path.join(sys_path, "make_tomo_config_geometry.py"))
        mk = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mk)
        assert mk.parse(root) == golden
    acq, _, _ = simul.workload("tomo_config_1024")
    g = Geometry.from_acquisition(acq)
    for k, v in golden.items():
        assert getattr(g, k) == v, k


def _read_hdf5(path):
    """A reader of the HDF5 structures the writer uses, after the format
    specification: superblock 0, the root group's symbol table (local heap,
    version-1 B-tree of group nodes, symbol table nodes), object headers of
    version 1 and their dataspace, datatype and layout messages.  Returns
    {group path: {dataset name: array}}."""
    buf = open(path, "rb").read()
    assert buf[:8] == b"\x89HDF\r\n\x1a\n"
    assert buf[8] == 0 and buf[13] == 8 and buf[14] == 8          # superblock 0, 8-byte offsets and lengths
    leaf_k, node_k = struct.unpack_from("<HH", buf, 16)
    eof = struct.unpack_from("<Q", buf, 40)[0]
    assert eof == len(buf)

    def messages(addr):
        ver, _, nmsg, _, size, _ = struct.unpack_from("<BBHIII", buf, addr)
        assert ver == 1
        out, at = [], addr + 16
        for _ in range(nmsg):
            typ, sz, _flags = struct.unpack_from("<HHB", buf, at)
            out.append((typ, buf[at + 8:at + 8 + sz]))
            at += 8 + sz
        assert at == addr + 16 + size
        return out

    def heap_name(heap, off):
        assert buf[heap:heap + 4] == b"HEAP"
        assert struct.unpack_from("<Q", buf, heap + 16)[0] == 1   # no free block
        data = struct.unpack_from("<Q", buf, heap + 24)[0]
        end = buf.index(b"\0", data + off)
        return buf[data + off:end].decode()

    def members(btree, heap):
        assert buf[btree:btree + 4] == b"TREE" and buf[btree + 4] == 0 and buf[btree + 5] == 0
        used = struct.unpack_from("<H", buf, btree + 6)[0]
        out = {}
        for c in range(used):
            snod = struct.unpack_from("<Q", buf, btree + 24 + 8 + 16 * c)[0]
            assert buf[snod:snod + 4] == b"SNOD" and buf[snod + 4] == 1
            nsym = struct.unpack_from("<H", buf, snod + 6)[0]
            assert nsym <= 2 * leaf_k
            for e in range(nsym):
                name_off, ohdr = struct.unpack_from("<QQ", buf, snod + 8 + 40 * e)
                out[heap_name(heap, name_off)] = ohdr
        return out

    def read_object(ohdr):
        msgs = dict(messages(ohdr))
        if 0x0011 in msgs:
            bt, hp = struct.unpack("<QQ", msgs[0x0011])
            return {n: read_object(a) for n, a in members(bt, hp).items()}
        sp, ty, lay = msgs[0x0001], msgs[0x0003], msgs[0x0008]
        assert 0x0005 in msgs
        rank = sp[1]
        dims = struct.unpack_from("<" + "Q" * rank, sp, 8)
        assert ty[0] == 0x11 and struct.unpack_from("<I", ty, 4)[0] == 4   # IEEE float, 4 bytes
        assert (ty[1] & 1) == 0 and ty[2] == 31                            # little endian, sign bit 31
        assert lay[0] == 3 and lay[1] == 1                                 # contiguous
        addr, size = struct.unpack_from("<QQ", lay, 2)
        assert size == 4 * int(np.prod(dims))
        return np.frombuffer(buf, "<f4", int(np.prod(dims)), addr).reshape(dims)

    root_ohdr = struct.unpack_from("<Q", buf, 56 + 8)[0]
    return read_object(root_ohdr)


def test_hdf5_complex_volume(tmp_path):
    """The polarisation mode's output: /indice_complexe/Re and /Im, float32
    (nz, ny, nx), read back through the format's own structures."""
    rng = np.random.default_rng(3)
    re = rng.standard_normal((5, 6, 7)).astype(np.float32)
    im = rng.standard_normal((5, 6, 7)).astype(np.float32)
    p = str(tmp_path / "indice_cplx_hdf5.hdf")
    api.write_hdf5_complex(p, re, im)
    tree = _read_hdf5(p)
    assert set(tree) == {"indice_complexe"} and set(tree["indice_complexe"]) == {"Re", "Im"}
    np.testing.assert_array_equal(tree["indice_complexe"]["Re"], re)
    np.testing.assert_array_equal(tree["indice_complexe"]["Im"], im)
