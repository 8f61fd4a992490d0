"""Cholesky-integral files of the reference (`FCIDUMP_chol`, written by
ad_afqmc/pyscf_interface.py:578-598 `write_dqmc` with h5py, read by
ad_afqmc/mpi_jax.py:39-60 `_prep_afqmc`), without h5py.

The file is HDF5: datasets "header" = [nelec, nmo, ms, nchol] (int64), "hcore",
"hcore_mod", "chol" (flattened float64), "energy_core" (scalar), and optionally
"mo_coeffs_up" / "mo_coeffs_dn". h5py is not part of this environment, so this module
carries a small reader for the subset of HDF5 such files use (superblock version 0,
version-1 object headers, symbol-table groups with a version-1 B-tree and a local heap,
contiguous or compact datasets of little- or big-endian integers and IEEE floats) and a
writer of the same subset, following the published HDF5 file-format specification.

`ham_data_from_fcidump` turns a file into the inputs of the hot path, as `_prep_afqmc`
does: h0, h1 [2, nmo, nmo], chol [nchol, nmo * nmo], the electron counts per spin from
(nelec, ms), and the trial orbitals when the file has them.
"""

from __future__ import annotations

import struct
from typing import Dict, Optional

import numpy as np

_SIG = b"\x89HDF\r\n\x1a\n"
_UNDEF = 0xFFFFFFFFFFFFFFFF


class H5FormatError(ValueError):
    pass


# ----------------------------------------------------------------------------------------
# reader
# ----------------------------------------------------------------------------------------


class _Reader:
    def __init__(self, data: bytes):
        if data[:8] != _SIG:
            raise H5FormatError("not an HDF5 file")
        self.d = data
        if data[8] != 0:
            raise H5FormatError(f"superblock version {data[8]} (only version 0 is read)")
        self.so, self.sl = data[13], data[14]
        if self.so != 8 or self.sl != 8:
            raise H5FormatError("only 8-byte offsets and lengths are read")
        # root group symbol table entry after base, free-space, EOF and driver addresses
        self.root = self._entry(24 + 4 * 8)

    def u(self, off: int, n: int) -> int:
        return int.from_bytes(self.d[off:off + n], "little")

    def _entry(self, off: int) -> dict:
        return {"name_off": self.u(off, 8), "header": self.u(off + 8, 8), "cache": self.u(off + 16, 4),
                "scratch": self.d[off + 24:off + 40]}

    def messages(self, addr: int):
        """(type, body) of every message of the version-1 object header at addr."""
        d = self.d
        if d[addr] != 1:
            raise H5FormatError(f"object header version {d[addr]} (only version 1 is read)")
        nmsg = self.u(addr + 2, 2)
        size = self.u(addr + 8, 4)
        blocks = [(addr + 16, size)]
        out = []
        while blocks and len(out) < nmsg:
            start, length = blocks.pop(0)
            p = start
            while p + 8 <= start + length and len(out) < nmsg:
                mtype, msize = self.u(p, 2), self.u(p + 2, 2)
                body = d[p + 8:p + 8 + msize]
                if mtype == 0x10:  # continuation: more messages elsewhere
                    blocks.append((int.from_bytes(body[0:8], "little"), int.from_bytes(body[8:16], "little")))
                out.append((mtype, body))
                p += 8 + msize
        return out

    def group_entries(self, header_addr: int, scratch: Optional[bytes] = None) -> Dict[str, int]:
        btree = heap = None
        for mtype, body in self.messages(header_addr):
            if mtype == 0x11:
                btree, heap = int.from_bytes(body[0:8], "little"), int.from_bytes(body[8:16], "little")
        if btree is None and scratch is not None:
            btree, heap = int.from_bytes(scratch[0:8], "little"), int.from_bytes(scratch[8:16], "little")
        if btree is None:
            raise H5FormatError("group without a symbol table")
        if self.d[heap:heap + 4] != b"HEAP":
            raise H5FormatError("bad local heap")
        heap_data = self.u(heap + 24, 8)
        names: Dict[str, int] = {}
        self._walk_btree(btree, heap_data, names)
        return names

    def _walk_btree(self, addr: int, heap_data: int, names: Dict[str, int]) -> None:
        d = self.d
        if d[addr:addr + 4] != b"TREE" or d[addr + 4] != 0:
            raise H5FormatError("bad group B-tree node")
        level, used = d[addr + 5], self.u(addr + 6, 2)
        p = addr + 24 + 8  # after the header and key 0
        for _ in range(used):
            child = self.u(p, 8)
            p += 16  # child, next key
            if level > 0:
                self._walk_btree(child, heap_data, names)
                continue
            if d[child:child + 4] != b"SNOD":
                raise H5FormatError("bad symbol table node")
            for i in range(self.u(child + 6, 2)):
                e = self._entry(child + 8 + 40 * i)
                nm = d[heap_data + e["name_off"]:d.index(b"\0", heap_data + e["name_off"])].decode()
                names[nm] = e["header"]

    def dataset(self, header_addr: int) -> np.ndarray:
        shape = dtype = raw = None
        for mtype, b in self.messages(header_addr):
            if mtype == 0x01:  # dataspace
                ver, rank = b[0], b[1]
                if ver == 1:
                    shape = tuple(int.from_bytes(b[8 + 8 * i:16 + 8 * i], "little") for i in range(rank))
                elif ver == 2:
                    shape = () if b[3] == 0 else tuple(
                        int.from_bytes(b[4 + 8 * i:12 + 8 * i], "little") for i in range(rank))
                else:
                    raise H5FormatError(f"dataspace version {ver}")
            elif mtype == 0x03:  # datatype
                cls, size, bits = b[0] & 0x0F, int.from_bytes(b[4:8], "little"), b[1]
                order = ">" if bits & 1 else "<"
                if cls == 0:
                    dtype = np.dtype(f"{order}{'i' if bits & 0x08 else 'u'}{size}")
                elif cls == 1:
                    dtype = np.dtype(f"{order}f{size}")
                else:
                    raise H5FormatError(f"datatype class {cls} is not read")
            elif mtype == 0x08:  # data layout
                ver, lcls = b[0], b[1]
                if ver != 3:
                    raise H5FormatError(f"data layout version {ver}")
                if lcls == 0:
                    n = int.from_bytes(b[2:4], "little")
                    raw = b[4:4 + n]
                elif lcls == 1:
                    addr, n = int.from_bytes(b[2:10], "little"), int.from_bytes(b[10:18], "little")
                    raw = b"" if addr == _UNDEF else self.d[addr:addr + n]
                else:
                    raise H5FormatError("chunked datasets are not read")
        if shape is None or dtype is None or raw is None:
            raise H5FormatError("dataset without dataspace, datatype or layout")
        count = int(np.prod(shape)) if shape else 1
        if not raw:
            return np.zeros(shape, dtype=dtype.newbyteorder("="))
        return np.frombuffer(raw, dtype=dtype, count=count).reshape(shape).astype(dtype.newbyteorder("="))


def read_h5(path: str) -> Dict[str, np.ndarray]:
    """Every dataset of the root group of an HDF5 file (the subset described above)."""
    with open(path, "rb") as f:
        r = _Reader(f.read())
    names = r.group_entries(r.root["header"], r.root["scratch"] if r.root["cache"] == 1 else None)
    return {k: r.dataset(a) for k, a in sorted(names.items())}


# ----------------------------------------------------------------------------------------
# writer (same subset)
# ----------------------------------------------------------------------------------------


def _msg(mtype: int, body: bytes) -> bytes:
    body = body + b"\0" * ((-len(body)) % 8)
    return struct.pack("<HHB3x", mtype, len(body), 0) + body


def _header(msgs: bytes, nmsg: int) -> bytes:
    return struct.pack("<BBHII4x", 1, 0, nmsg, 1, len(msgs)) + msgs


def write_h5(path: str, datasets: Dict[str, np.ndarray]) -> None:
    """A root group of contiguous datasets (int64 / float64 arrays or scalars), readable by
    read_h5 and laid out as HDF5 files of superblock version 0."""
    items = sorted(datasets.items())
    if len(items) > 32:
        raise ValueError("at most 32 datasets")
    heap = bytearray(b"\0" * 8)  # offset 0: the empty name
    name_off = []
    for k, _ in items:
        name_off.append(len(heap))
        heap += k.encode() + b"\0"
        heap += b"\0" * ((-len(heap)) % 8)
    arrays = []
    for _, v in items:
        a = np.asarray(v)
        if a.dtype.kind in "iub":
            a = a.astype("<i8")
        elif a.dtype.kind == "f":
            a = a.astype("<f8")
        else:
            raise ValueError(f"dtype {a.dtype} is not written")
        arrays.append(np.array(a, order="C"))  # keeps 0-d arrays 0-d
    # layout: superblock (96) | root header | B-tree | SNOD | heap header | heap data |
    # dataset headers | raw data
    sb_size, leaf_k = 96, 16
    root_msgs = _msg(0x11, b"\0" * 16)  # patched below
    root_hdr_size = len(_header(root_msgs, 1))
    btree_size = 24 + 8 + 2 * 16 * (8 + 8)
    snod_size = 8 + 2 * leaf_k * 40
    heap_hdr_size = 32
    off = sb_size
    root_addr = off
    off += root_hdr_size
    btree_addr = off
    off += btree_size
    snod_addr = off
    off += snod_size
    heap_addr = off
    off += heap_hdr_size
    heap_data_addr = off
    off += len(heap)
    ds_addr = []
    for a in arrays:
        ds_addr.append(off)
        off += len(_header(_ds_msgs(a, 0), 3))
    raw_addr = []
    for a in arrays:
        off += (-off) % 8
        raw_addr.append(off)
        off += a.nbytes
    eof = off
    out = bytearray(eof)
    out[0:8] = _SIG
    out[8:24] = bytes([0, 0, 0, 0, 0, 8, 8, 0]) + struct.pack("<HHI", leaf_k, 16, 0)
    out[24:56] = struct.pack("<QQQQ", 0, _UNDEF, eof, _UNDEF)
    out[56:96] = struct.pack("<QQII", 0, root_addr, 1, 0) + struct.pack("<QQ", btree_addr, heap_addr)
    root = _header(_msg(0x11, struct.pack("<QQ", btree_addr, heap_addr)), 1)
    out[root_addr:root_addr + len(root)] = root
    last_key = name_off[-1] if name_off else 0
    bt = b"TREE" + struct.pack("<BBHQQ", 0, 0, 1, _UNDEF, _UNDEF) + struct.pack("<QQQ", 0, snod_addr, last_key)
    out[btree_addr:btree_addr + len(bt)] = bt
    sn = b"SNOD" + struct.pack("<BBH", 1, 0, len(items))
    for no, da in zip(name_off, ds_addr):
        sn += struct.pack("<QQII", no, da, 0, 0) + b"\0" * 16
    out[snod_addr:snod_addr + len(sn)] = sn
    hh = b"HEAP" + struct.pack("<B3xQQQ", 0, len(heap), _UNDEF, heap_data_addr)
    out[heap_addr:heap_addr + len(hh)] = hh
    out[heap_data_addr:heap_data_addr + len(heap)] = heap
    for a, da, ra in zip(arrays, ds_addr, raw_addr):
        h = _header(_ds_msgs(a, ra), 3)
        out[da:da + len(h)] = h
        out[ra:ra + a.nbytes] = a.tobytes()
    with open(path, "wb") as f:
        f.write(bytes(out))


def _ds_msgs(a: np.ndarray, raw_addr: int) -> bytes:
    space = struct.pack("<BBB5x", 1, a.ndim, 0) + b"".join(struct.pack("<Q", s) for s in a.shape)
    if a.dtype.kind == "i":  # signed 64-bit little-endian integer
        dtype = struct.pack("<BBBBIHH", 0x10, 0x08, 0, 0, 8, 0, 64)
    else:  # IEEE float64 little-endian
        dtype = struct.pack("<BBBBIHHBBBBI", 0x11, 0x20, 0x3F, 0, 8, 0, 64, 52, 11, 0, 52, 1023)
    layout = struct.pack("<BBQQ", 3, 1, raw_addr, a.nbytes)
    return _msg(0x01, space) + _msg(0x03, dtype) + _msg(0x08, layout)


# ----------------------------------------------------------------------------------------
# FCIDUMP_chol
# ----------------------------------------------------------------------------------------


def read_fcidump_chol(path: str) -> dict:
    """The fields of a Cholesky-integral file, shaped as _prep_afqmc uses them
    (mpi_jax.py:39-60): nelec, nmo, ms, nchol, h0, h1 [nmo, nmo], h1_mod, chol
    [nchol, nmo, nmo], and mo_coeffs [up, dn] when present."""
    f = read_h5(path)
    nelec, nmo, ms, nchol = (int(x) for x in f["header"])
    out = {"nelec": nelec, "nmo": nmo, "ms": ms, "nchol": nchol,
           "h0": float(np.asarray(f["energy_core"]).reshape(-1)[0]),
           "h1": np.asarray(f["hcore"], dtype=np.float64).reshape(nmo, nmo),
           "h1_mod": np.asarray(f["hcore_mod"], dtype=np.float64).reshape(nmo, nmo),
           "chol": np.asarray(f["chol"], dtype=np.float64).reshape(-1, nmo, nmo)}
    if "mo_coeffs_up" in f:
        out["mo_coeffs"] = [np.asarray(f["mo_coeffs_up"]), np.asarray(f["mo_coeffs_dn"])]
    return out


def write_fcidump_chol(path: str, hcore, hcore_mod, chol, nelec: int, nmo: int, enuc: float, ms: int = 0,
                       mo_coeffs=None) -> None:
    """The file write_dqmc produces (pyscf_interface.py:578-598), with this module's writer."""
    chol = np.asarray(chol)
    d = {"header": np.array([nelec, nmo, ms, chol.shape[0]], dtype=np.int64),
         "hcore": np.asarray(hcore, dtype=np.float64).reshape(-1),
         "hcore_mod": np.asarray(hcore_mod, dtype=np.float64).reshape(-1),
         "chol": chol.astype(np.float64).reshape(-1), "energy_core": np.float64(enuc)}
    if mo_coeffs is not None:
        d["mo_coeffs_up"] = np.asarray(mo_coeffs[0], dtype=np.float64)
        d["mo_coeffs_dn"] = np.asarray(mo_coeffs[1], dtype=np.float64)
    write_h5(path, d)


def ham_data_from_fcidump(path: str) -> dict:
    """ham_data (h0, h1 [2, nmo, nmo], chol [nchol, nmo * nmo], ene0 = 0) plus norb and the
    electron counts per spin, nelec_sp = ((nelec + |ms|) // 2, (nelec - |ms|) // 2), as
    _prep_afqmc builds them (mpi_jax.py:39-60); "mo_coeff" when the file has trial orbitals."""
    f = read_fcidump_chol(path)
    nmo, ms, nelec = f["nmo"], f["ms"], f["nelec"]
    out = {"ham_data": {"h0": f["h0"], "h1": np.stack([f["h1"], f["h1"]]),
                        "chol": f["chol"].reshape(f["chol"].shape[0], nmo * nmo), "ene0": 0.0},
           "norb": nmo, "nelec": ((nelec + abs(ms)) // 2, (nelec - abs(ms)) // 2), "nchol": f["nchol"]}
    if "mo_coeffs" in f:
        out["mo_coeff"] = f["mo_coeffs"]
    return out
