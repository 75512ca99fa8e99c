"""Cells of the first worksheet of an Excel 97-2003 (.xls) workbook, the
format xdynamics model files use (read there through BasicExcel,
source/xXLSReader.cpp:354-361, sheet 0 only).

Written from the published formats: the OLE2 compound file (a FAT of
sector chains, a directory of 128-byte entries, streams below 4096 bytes in
the mini stream) holding the "Workbook" stream, and the BIFF8 records in
it.  The cell records read are LABELSST (shared string table SST, split by
CONTINUE records), LABEL, NUMBER, RK, MULRK and FORMULA (its cached number,
or the STRING record after it).  Other records are skipped.

    cells = read_cells(path)      # {(row, col): str or float}, zero-based
"""
import struct

_SIG = b"\xd0\xcf\x11\xe0\xa1\xb1\x1a\xe1"
_FREE, _END = 0xFFFFFFFF, 0xFFFFFFFE


class XlsError(ValueError):
    pass


def _stream(data, name_wanted=("Workbook", "Book")):
    if data[:8] != _SIG:
        raise XlsError("not an OLE2 compound file")
    sec_shift, mini_shift = struct.unpack_from("<HH", data, 0x1E)
    ssz, mssz = 1 << sec_shift, 1 << mini_shift
    n_fat, dir_start = struct.unpack_from("<II", data, 0x2C)
    mini_cutoff, minifat_start, n_minifat, difat_start, n_difat = struct.unpack_from("<IIIII", data, 0x38)

    def sector(i):
        off = (i + 1) * ssz
        if off >= len(data):
            raise XlsError(f"sector {i} beyond the file")
        return data[off:off + ssz]

    difat = list(struct.unpack_from("<109I", data, 0x4C))
    d = difat_start
    for _ in range(n_difat):
        if d in (_FREE, _END):
            break
        ent = struct.unpack(f"<{ssz // 4}I", sector(d))
        difat.extend(ent[:-1])
        d = ent[-1]
    fat = []
    for s in difat[:n_fat]:
        fat.extend(struct.unpack(f"<{ssz // 4}I", sector(s)))

    def chain(start, table):
        out, i, seen = [], start, 0
        while i not in (_FREE, _END):
            if i >= len(table) or seen > len(table):
                raise XlsError("broken sector chain")
            out.append(i)
            i = table[i]
            seen += 1
        return out

    dir_bytes = b"".join(sector(i) for i in chain(dir_start, fat))
    entries = []
    for off in range(0, len(dir_bytes) - 127, 128):
        e = dir_bytes[off:off + 128]
        nlen = struct.unpack_from("<H", e, 0x40)[0]
        name = e[:max(nlen - 2, 0)].decode("utf-16-le", errors="replace")
        typ = e[0x42]
        start, size = struct.unpack_from("<II", e, 0x74)
        entries.append((name, typ, start, size))
    root = next((e for e in entries if e[1] == 5), None)
    if root is None:
        raise XlsError("no root entry")
    minifat = []
    for s in chain(minifat_start, fat) if n_minifat else []:
        minifat.extend(struct.unpack(f"<{ssz // 4}I", sector(s)))
    mini_stream = b"".join(sector(i) for i in chain(root[2], fat)) if root[2] not in (_FREE, _END) else b""
    for name, typ, start, size in entries:
        if typ == 2 and name in name_wanted:
            if size < mini_cutoff:
                buf = b"".join(mini_stream[i * mssz:(i + 1) * mssz] for i in chain(start, minifat))
            else:
                buf = b"".join(sector(i) for i in chain(start, fat))
            return buf[:size]
    raise XlsError("no Workbook stream")


def _records(wb, start=0):
    off = start
    while off + 4 <= len(wb):
        rtype, rlen = struct.unpack_from("<HH", wb, off)
        yield off, rtype, wb[off + 4:off + 4 + rlen]
        off += 4 + rlen


def _rk(v):
    if v & 2:
        x = v >> 2
        if x & (1 << 29):
            x -= 1 << 30
        x = float(x)
    else:
        x = struct.unpack("<d", struct.pack("<Q", (v & 0xFFFFFFFC) << 32))[0]
    return x / 100.0 if v & 1 else x


class _Chunks:
    """Reads across an SST record and its CONTINUE records: a string's
    characters may cross a record boundary, where a new option byte says
    whether the rest is 8- or 16-bit."""

    def __init__(self, parts):
        self.parts = parts
        self.i = 0
        self.off = 0

    def left(self):
        return len(self.parts[self.i]) - self.off

    def advance_part(self):
        if self.i + 1 >= len(self.parts):
            raise XlsError("shared string table ends early")
        self.i += 1
        self.off = 0

    def take(self, n):
        out = b""
        while n > 0:
            if self.left() == 0:
                self.advance_part()
            k = min(n, self.left())
            out += self.parts[self.i][self.off:self.off + k]
            self.off += k
            n -= k
        return out

    def chars(self, n, wide):
        s = []
        while n > 0:
            if self.left() == 0:
                self.advance_part()
                wide = bool(self.take(1)[0] & 1)
            w = 2 if wide else 1
            k = min(n, self.left() // w)
            raw = self.take(k * w)
            s.append(raw.decode("utf-16-le") if wide else raw.decode("latin-1"))
            n -= k
        return "".join(s)


def _sst(parts):
    c = _Chunks(parts)
    total, unique = struct.unpack("<II", c.take(8))
    out = []
    for _ in range(unique):
        n = struct.unpack("<H", c.take(2))[0]
        flags = c.take(1)[0]
        runs = struct.unpack("<H", c.take(2))[0] if flags & 8 else 0
        ext = struct.unpack("<I", c.take(4))[0] if flags & 4 else 0
        out.append(c.chars(n, bool(flags & 1)))
        c.take(4 * runs + ext)
    return out


def _label(data, off):
    n = struct.unpack_from("<H", data, off)[0]
    flags = data[off + 2]
    raw = data[off + 3:]
    return raw[:2 * n].decode("utf-16-le") if flags & 1 else raw[:n].decode("latin-1")


def read_cells(path, sheet=0):
    """{(row, col): value} of worksheet `sheet` (zero-based indices; strings
    as str, numbers as float)."""
    wb = _stream(open(path, "rb").read())
    sheets, sst = [], []
    recs = list(_records(wb))
    for k, (off, rtype, data) in enumerate(recs):
        if rtype == 0x0085:      # BOUNDSHEET
            sheets.append(struct.unpack_from("<I", data, 0)[0])
        elif rtype == 0x00FC:    # SST and its CONTINUE records
            parts = [data]
            j = k + 1
            while j < len(recs) and recs[j][1] == 0x003C:
                parts.append(recs[j][2])
                j += 1
            sst = _sst(parts)
        elif rtype == 0x000A and sheets:  # EOF of the globals
            break
    if sheet >= len(sheets):
        raise XlsError(f"workbook has {len(sheets)} sheets")
    cells = {}
    pending = None
    for off, rtype, data in _records(wb, sheets[sheet]):
        if rtype == 0x000A:      # EOF of the sheet
            break
        if rtype == 0x00FD:      # LABELSST
            r, c, _, i = struct.unpack_from("<HHHI", data, 0)
            cells[(r, c)] = sst[i]
        elif rtype == 0x0204:    # LABEL
            r, c, _ = struct.unpack_from("<HHH", data, 0)
            cells[(r, c)] = _label(data, 6)
        elif rtype == 0x0203:    # NUMBER
            r, c, _, v = struct.unpack_from("<HHHd", data, 0)
            cells[(r, c)] = v
        elif rtype == 0x027E:    # RK
            r, c, _, v = struct.unpack_from("<HHHI", data, 0)
            cells[(r, c)] = _rk(v)
        elif rtype == 0x00BD:    # MULRK
            r, c0 = struct.unpack_from("<HH", data, 0)
            n = (len(data) - 6) // 6
            for i in range(n):
                v = struct.unpack_from("<I", data, 4 + 6 * i + 2)[0]
                cells[(r, c0 + i)] = _rk(v)
        elif rtype == 0x0006:    # FORMULA: cached result
            r, c, _ = struct.unpack_from("<HHH", data, 0)
            res = data[6:14]
            if res[6:8] == b"\xff\xff":
                if res[0] == 0:
                    pending = (r, c)  # string in the STRING record that follows
            else:
                cells[(r, c)] = struct.unpack("<d", res)[0]
        elif rtype == 0x0207 and pending:  # STRING
            cells[pending] = _label(data, 0)
            pending = None
    return cells
