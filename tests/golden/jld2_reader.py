"""Minimal reader for the reference's JLD2 test fixtures (HDF5 subset).

Used only by make_goldens.py, at fixture-generation time, to read the
integrals, clusters, Fock sectors and densities stored in the reference's
test/_testdata_*.jld2 files (h5py is not available).  It understands what
JLD2 0.1.x writes for those files: superblock v2/v3, version-2 object headers
(with continuation blocks), link / dataspace / datatype / layout / attribute
messages, committed (shared) datatypes, compound / float / integer /
reference / variable-length datatypes, compact and contiguous storage.
Julia arrays come back in Julia's index order (HDF5 dims are reversed).
"""
from __future__ import annotations

import struct

import numpy as np


class JLD2File:
    def __init__(self, path):
        self.d = open(path, "rb").read()
        sig = b"\x89HDF\r\n\x1a\n"
        self.base = None
        for off in (0, 512, 1024, 2048, 4096):
            if self.d[off:off + 8] == sig:
                self.base = off
                break
        if self.base is None:
            raise ValueError("no HDF5 superblock")
        sb = self.base
        ver = self.d[sb + 8]
        if ver not in (2, 3):
            raise ValueError(f"superblock version {ver} unsupported")
        so, sl = self.d[sb + 9], self.d[sb + 10]
        assert so == 8 and sl == 8
        # base addr, ext addr, eof addr, root obj header addr
        self.root = struct.unpack_from("<Q", self.d, sb + 12 + 24)[0]
        self._dtcache = {}

    # ---- object headers ---------------------------------------------------------------
    def messages(self, addr):
        d = self.d
        p = self.base + addr
        if d[p:p + 4] != b"OHDR":
            raise ValueError(f"no OHDR at {addr:#x}")
        flags = d[p + 5]
        q = p + 6
        if flags & 0x20:
            q += 16
        if flags & 0x10:
            q += 4
        szlen = 1 << (flags & 3)
        size = int.from_bytes(d[q:q + szlen], "little")
        q += szlen
        blocks = [(q, q + size)]
        out = []
        crt = bool(flags & 0x04)
        while blocks:
            s, e = blocks.pop(0)
            while s + 4 <= e:
                mtype = d[s]
                msize = struct.unpack_from("<H", d, s + 1)[0]
                mflags = d[s + 3]
                s += 4 + (2 if crt else 0)
                body = d[s:s + msize]
                s += msize
                if mtype == 0x10:  # continuation
                    caddr, clen = struct.unpack_from("<QQ", body, 0)
                    cp = self.base + caddr
                    assert d[cp:cp + 4] == b"OCHK"
                    blocks.append((cp + 4, cp + clen - 4))
                elif mtype != 0:
                    out.append((mtype, mflags, body))
        return out

    def links(self, addr):
        res = {}
        for t, f, b in self.messages(addr):
            if t != 6:
                continue
            fl = b[1]
            q = 2
            ltype = 0
            if fl & 0x08:
                ltype = b[q]
                q += 1
            if fl & 0x04:
                q += 8
            if fl & 0x10:
                q += 1
            ln = 1 << (fl & 3)
            nlen = int.from_bytes(b[q:q + ln], "little")
            q += ln
            name = b[q:q + nlen].decode()
            q += nlen
            if ltype == 0:
                res[name] = struct.unpack_from("<Q", b, q)[0]
        return res

    # ---- datatypes -------------------------------------------------------------------------
    def datatype(self, body, off=0):
        """Parse a datatype message at body[off:]; returns (dtype dict, bytes consumed)."""
        cv = body[off]
        cls, ver = cv & 0x0F, cv >> 4
        bits = body[off + 1:off + 4]
        size = struct.unpack_from("<I", body, off + 4)[0]
        q = off + 8
        if cls == 0:  # fixed point
            signed = bool(bits[0] & 0x08)
            q += 4
            return {"class": "int", "size": size, "signed": signed}, q - off
        if cls == 1:  # float
            q += 12
            return {"class": "float", "size": size}, q - off
        if cls == 3:  # string
            return {"class": "string", "size": size}, q - off
        if cls == 7:  # reference
            return {"class": "ref", "size": size}, q - off
        if cls == 9:  # variable length
            base, n = self.datatype(body, q)
            return {"class": "vlen", "size": size, "base": base, "is_string": (bits[0] & 0x0F) == 1}, q + n - off
        if cls == 6:  # compound
            nmem = struct.unpack_from("<H", bits, 0)[0]
            mems = []
            for _ in range(nmem):
                e = body.index(b"\x00", q)
                name = body[q:e].decode()
                if ver < 3:
                    q = e + 1
                    q = q + ((8 - (q - off) % 8) % 8) if False else q
                    raise ValueError("compound version < 3 unsupported")
                q = e + 1
                ob = 1 if size < 256 else 2 if size < 65536 else 4
                moff = int.from_bytes(body[q:q + ob], "little")
                q += ob
                mt, n = self.datatype(body, q)
                q += n
                mems.append((name, moff, mt))
            return {"class": "compound", "size": size, "members": mems}, q - off
        if cls == 10:  # array
            nd = body[q]
            q += 1
            dims = struct.unpack_from("<" + "I" * nd, body, q)
            q += 4 * nd
            base, n = self.datatype(body, q)
            return {"class": "array", "size": size, "dims": dims, "base": base}, q + n - off
        raise ValueError(f"datatype class {cls} unsupported")

    def _dtype_of(self, msgs):
        for t, f, b in msgs:
            if t == 3:
                if f & 0x02:  # shared (committed) datatype
                    addr = struct.unpack_from("<Q", b, 2)[0]
                    if addr not in self._dtcache:
                        inner = [m for m in self.messages(addr) if m[0] == 3][0]
                        self._dtcache[addr] = self.datatype(inner[2])[0]
                    return self._dtcache[addr]
                return self.datatype(b)[0]
        return None

    # ---- datasets -------------------------------------------------------------------------
    def _dataspace(self, msgs):
        for t, f, b in msgs:
            if t == 1:
                ver, nd, fl = b[0], b[1], b[2]
                if ver == 1:
                    q = 8
                else:
                    stype = b[3]
                    q = 4
                    if stype == 2:
                        return None
                dims = struct.unpack_from("<" + "Q" * nd, b, q)
                return tuple(dims)
        return ()

    def _raw(self, msgs, nbytes):
        for t, f, b in msgs:
            if t == 8:
                ver = b[0]
                cls = b[1]
                if cls == 0:
                    sz = struct.unpack_from("<H", b, 2)[0]
                    return b[4:4 + sz]
                if cls == 1:
                    addr, sz = struct.unpack_from("<QQ", b, 2)
                    return self.d[self.base + addr:self.base + addr + sz]
                raise ValueError("chunked storage unsupported")
        raise ValueError("no layout message")

    def read(self, addr):
        msgs = self.messages(addr)
        dt = self._dtype_of(msgs)
        dims = self._dataspace(msgs)
        if dims is None:  # null dataspace: singleton / empty struct
            return None
        n = int(np.prod(dims)) if dims else 1
        raw = self._raw(msgs, n * dt["size"])
        vals = [self.decode(dt, raw, i * dt["size"]) for i in range(n)]
        if not dims:
            return vals[0]
        if dt["class"] in ("float", "int"):
            arr = np.array(vals).reshape(dims)
            return np.transpose(arr, tuple(range(len(dims) - 1, -1, -1)))
        return np.array(vals, dtype=object).reshape(dims[::-1], order="F") if len(dims) > 1 else vals

    def decode(self, dt, raw, off):
        c = dt["class"]
        if c == "float":
            return struct.unpack_from("<d" if dt["size"] == 8 else "<f", raw, off)[0]
        if c == "int":
            fmt = {1: "b", 2: "h", 4: "i", 8: "q"}[dt["size"]]
            if not dt["signed"]:
                fmt = fmt.upper()
            return struct.unpack_from("<" + fmt, raw, off)[0]
        if c == "ref":
            a = struct.unpack_from("<Q", raw, off)[0]
            return self.read(a) if a else None
        if c == "compound":
            return {name: self.decode(mt, raw, off + mo) for name, mo, mt in dt["members"]}
        if c == "array":
            n = int(np.prod(dt["dims"]))
            bs = dt["base"]["size"]
            return [self.decode(dt["base"], raw, off + i * bs) for i in range(n)]
        if c == "vlen":
            length, heap, idx = struct.unpack_from("<IQI", raw, off)
            data = self._global_heap(heap, idx)
            if dt["is_string"]:
                return data.decode()
            bs = dt["base"]["size"]
            return [self.decode(dt["base"], data, i * bs) for i in range(length)]
        if c == "string":
            return raw[off:off + dt["size"]].split(b"\x00")[0].decode()
        raise ValueError(c)

    def _global_heap(self, addr, idx):
        p = self.base + addr
        assert self.d[p:p + 4] == b"GCOL"
        size = struct.unpack_from("<Q", self.d, p + 8)[0]
        q = p + 16
        end = p + size
        while q + 16 <= end:
            hidx, rc = struct.unpack_from("<HH", self.d, q)
            osz = struct.unpack_from("<Q", self.d, q + 8)[0]
            if hidx == idx:
                return self.d[q + 16:q + 16 + osz]
            if hidx == 0:
                break
            q += 16 + ((osz + 7) // 8) * 8
        raise KeyError(idx)

    def __getitem__(self, name):
        return self.read(self.links(self.root)[name])

    def keys(self):
        return list(self.links(self.root))
