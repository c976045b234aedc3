"""The iterate stage's input formats: the stdin parameter file and the data files.

* Parameter file: read by ``myReadOSB`` (``src/iterate/module/osb.print.h:192-246``)
  with Fortran list-directed reads, one read statement per group.
* ``H0``: ``loadData`` (``src/libutil/serial/io/io.f90:98-123``), Fortran unformatted
  *sequential* access: one record of doubles framed by 4-byte length markers
  (gfortran/ifort default; records over 2 GiB are split into sub-records whose
  leading marker is negative when another sub-record follows).
* ``RES``, ``DEP``, ``EIG``, ``OUTH``: ``loadDataDir`` (``src/libutil/serial/io/iodirect.f90:68-90``),
  direct access, one record of raw doubles, no markers.

Sizes follow ``calOSB`` (``src/iterate/module/osb.init.h:2-49``).
"""
from __future__ import annotations

import dataclasses
import struct

import numpy as np

FMAX = 20

# Preconditioner kinds (sOSB) and operator kinds (sHC/sPC): src/iterate/module/osb.data.h:10-20.
TOSB, TOSBD1, TOSBD2, TOSBW = 1, 2, 3, 4
JOB_BOUND = 1
JOB_RES1, JOB_RES2, JOB_CRP, JOB_CRP1, JOB_CRP2 = 2, 3, 4, 5, 6   # osb.data.h:13-14
TA0, TA1 = 0, 1


@dataclasses.dataclass
class OSBInput:
    """Everything ``myReadOSB`` reads, with the reference's variable names."""

    sF: int = 3
    sN: tuple = (24, 32, 20)
    sDEP: tuple = (False, False, True)
    sJOB: int = JOB_BOUND
    sOSB: int = TOSB
    sCX: bool = False
    sNDVR: bool = False
    sST: bool = False
    sAP: bool = False
    sBJ: tuple = (20, 1e-4)              # (mMax, mTol) of the block-Jacobi sweeps
    sQMR: tuple = (2000, 1e-4)           # (mMax, mTol) of the QMR inner solve
    sConv: tuple = (0.0, 1e-8, 0, 5, 0, 20, 1)  # (mE0, mTol, mStart, mStep, mMax, mNum, mGap)
    sOSBW: tuple = (0.0, 0.0, 0.0, 0)    # (mE0, mDE, mBeta, mCnt)
    sHOSB: int = 0
    sVOSB: int = 0
    sHW: int = 0
    sVX: int = 0
    sPT: int = 0
    H0File: str = "H0.dat"
    RESFile: str = "RES.dat"
    OUTHFile: str = ""
    DEPFile: str = "DEP.dat"
    HOSBFile: str = ""
    VOSBFile: str = ""
    EigFile: str = ""
    HWFile: str = ""
    APPFile: str = ""
    APRFile: str = ""
    VXFile: str = ""
    PTFile: str = ""

    # -- sizes: calOSB (osb.init.h:2-49) -------------------------------------------
    @property
    def my_dim(self):
        d = [1]
        for i in range(self.sF - 1):
            d.append(d[-1] * self.sN[i])
        return tuple(d)

    @property
    def my_blk(self):
        b = [1] * self.sF
        for i in range(self.sF - 1, 0, -1):
            b[i - 1] = b[i] * self.sN[i]
        return tuple(b)

    @property
    def my_len(self) -> int:
        return self.my_blk[0] * self.sN[0]

    @property
    def h0_len(self) -> int:
        return sum(n * n for i, n in enumerate(self.sN[:self.sF])
                   if not (self.sNDVR and i == self.sF - 1))

    @property
    def dep_len(self) -> int:
        return sum(self.my_dim[i] for i in range(self.sF) if self.sDEP[i])


class _ListReader:
    """Fortran list-directed reads: each read starts on a fresh record (line),
    may continue over following lines, and drops what is left of its last line."""

    def __init__(self, text: str):
        self._lines = iter(text.splitlines())
        self._pending = []

    def _more(self) -> bool:
        line = next(self._lines)
        stop = line.find("/")
        if stop >= 0:
            line = line[:stop]
        self._pending.extend(t for t in line.split("!")[0].replace(",", " ").split() if t)
        return stop < 0

    def start(self):
        self._pending = []

    def take(self, count: int):
        while len(self._pending) < count:
            if not self._more() and len(self._pending) < count:
                raise ValueError("list-directed read ended by '/' before all values")
        out, self._pending = self._pending[:count], self._pending[count:]
        return out

    def read(self, count: int):
        self.start()
        return self.take(count)

    def line(self) -> str:
        self._pending = []
        return next(self._lines).strip()


def _logical(tok: str) -> bool:
    t = tok.strip().lstrip(".").upper()
    if not t:
        raise ValueError("empty logical")
    if t[0] == "T":
        return True
    if t[0] == "F":
        return False
    raise ValueError(f"bad logical {tok!r}")


def _real(tok: str) -> float:
    return float(tok.upper().replace("D", "E"))


def read_input(text: str) -> OSBInput:
    """Parse a parameter file exactly in the order ``myReadOSB`` reads it."""
    rd = _ListReader(text)
    inp = OSBInput()
    rd.start()
    sF = int(rd.take(1)[0])
    if not (1 <= sF <= FMAX):
        raise ValueError(f"sF={sF} out of range 1..{FMAX}")
    inp.sF = sF
    inp.sN = tuple(int(v) for v in rd.take(sF))
    t = rd.read(sF)
    dep = [_logical(v) for v in t]
    dep[0] = False                                   # osb.print.h:198-199
    t = rd.read(2)
    inp.sJOB, inp.sOSB = int(t[0]), int(t[1])
    t = rd.read(4)
    inp.sCX, inp.sNDVR, inp.sST, inp.sAP = (_logical(v) for v in t)
    if inp.sNDVR:
        dep[sF - 1] = False
    inp.sDEP = tuple(dep)
    t = rd.read(4)
    inp.sBJ = (int(t[0]), _real(t[1]))
    inp.sQMR = (int(t[2]), _real(t[3]))
    t = rd.read(7)
    inp.sConv = (_real(t[0]), _real(t[1]), int(t[2]), int(t[3]), int(t[4]), int(t[5]), int(t[6]))
    t = rd.read(4)
    inp.sOSBW = (_real(t[0]), abs(_real(t[1])), _real(t[2]), int(t[3]))
    t = rd.read(5)
    inp.sHOSB, inp.sVOSB, inp.sHW, inp.sVX, inp.sPT = (int(v) for v in t)

    def name():
        return rd.line()

    inp.H0File = name()
    if inp.sNDVR:
        inp.OUTHFile = name()
    else:
        inp.RESFile = name()
    if any(inp.sDEP[:sF]):
        inp.DEPFile = name()
    if inp.sJOB in (JOB_RES1, JOB_RES2):                      # osb.print.h:230-231
        inp.APPFile = name()
    elif inp.sJOB in (JOB_CRP, JOB_CRP1, JOB_CRP2):           # osb.print.h:232-234
        inp.APPFile = name()
        inp.APRFile = name()
    if inp.sHOSB != 0:
        inp.HOSBFile = name()
    if inp.sVOSB != 0:
        inp.VOSBFile = name()
        inp.EigFile = name()
    if inp.sHW != 0:
        inp.HWFile = name()
    if inp.sVX != 0:
        inp.VXFile = name()
    if inp.sPT != 0:
        inp.PTFile = name()
    return inp


def _fmt_logical(b: bool) -> str:
    return "T" if b else "F"


def write_input(inp: OSBInput) -> str:
    """Render an :class:`OSBInput` as a parameter file ``read_input`` accepts."""
    out = []
    out.append(f"{inp.sF} " + " ".join(str(n) for n in inp.sN[:inp.sF]))
    out.append(" ".join(_fmt_logical(b) for b in inp.sDEP[:inp.sF]))
    out.append(f"{inp.sJOB} {inp.sOSB}")
    out.append(" ".join(_fmt_logical(b) for b in (inp.sCX, inp.sNDVR, inp.sST, inp.sAP)))
    out.append(f"{inp.sBJ[0]} {inp.sBJ[1]!r} {inp.sQMR[0]} {inp.sQMR[1]!r}")
    c = inp.sConv
    out.append(f"{c[0]!r} {c[1]!r} {c[2]} {c[3]} {c[4]} {c[5]} {c[6]}")
    w = inp.sOSBW
    out.append(f"{w[0]!r} {w[1]!r} {w[2]!r} {w[3]}")
    out.append(f"{inp.sHOSB} {inp.sVOSB} {inp.sHW} {inp.sVX} {inp.sPT}")
    out.append(inp.H0File)
    out.append(inp.OUTHFile if inp.sNDVR else inp.RESFile)
    if any(inp.sDEP[:inp.sF]):
        out.append(inp.DEPFile)
    if inp.sJOB in (JOB_RES1, JOB_RES2):
        out.append(inp.APPFile)
    elif inp.sJOB in (JOB_CRP, JOB_CRP1, JOB_CRP2):
        out.extend([inp.APPFile, inp.APRFile])
    for flag, names in ((inp.sHOSB, [inp.HOSBFile]), (inp.sVOSB, [inp.VOSBFile, inp.EigFile]),
                        (inp.sHW, [inp.HWFile]), (inp.sVX, [inp.VXFile]),
                        (inp.sPT, [inp.PTFile])):
        if flag != 0:
            out.extend(names)
    return "\n".join(out) + "\n"


# ----------------------------------------------------------------------------------
# data files
# ----------------------------------------------------------------------------------
_MAX_SUBRECORD = 2147483639  # gfortran's largest sub-record payload


def save_data(path, data: np.ndarray) -> None:
    """Write one unformatted sequential record (``saveData``/``loadData`` layout)."""
    buf = np.ascontiguousarray(data, dtype="<f8").tobytes()
    with open(path, "wb") as f:
        pos = 0
        n = len(buf)
        while True:
            chunk = buf[pos:pos + _MAX_SUBRECORD]
            more = pos + len(chunk) < n
            lead = -len(chunk) if more else len(chunk)
            trail = -len(chunk) if pos > 0 else len(chunk)
            f.write(struct.pack("<i", lead))
            f.write(chunk)
            f.write(struct.pack("<i", trail))
            pos += len(chunk)
            if not more:
                break


def save_records(path, records) -> None:
    """Several unformatted sequential records (bytes each), sub-records over 2 GiB."""
    with open(path, "wb") as f:
        for buf in records:
            pos, n = 0, len(buf)
            while True:
                chunk = buf[pos:pos + _MAX_SUBRECORD]
                more = pos + len(chunk) < n
                f.write(struct.pack("<i", -len(chunk) if more else len(chunk)))
                f.write(chunk)
                f.write(struct.pack("<i", -len(chunk) if pos > 0 else len(chunk)))
                pos += len(chunk)
                if not more:
                    break


def load_records(path):
    """All records of an unformatted sequential file as bytes."""
    out = []
    with open(path, "rb") as f:
        while True:
            hdr = f.read(4)
            if not hdr:
                return out
            rec = bytearray()
            while True:
                if len(hdr) != 4:
                    raise ValueError(f"{path}: truncated record marker")
                lead = struct.unpack("<i", hdr)[0]
                chunk = f.read(abs(lead))
                if len(chunk) != abs(lead) or len(f.read(4)) != 4:
                    raise ValueError(f"{path}: truncated record")
                rec += chunk
                if lead >= 0:
                    break
                hdr = f.read(4)
            out.append(bytes(rec))


def save_pist_basis(path, cnt, ritz, hmat, vj) -> None:
    """The PT file of PISTF_CONV (src/iterate/libiterate/pist/pistf.f90:98-104):
    (cnt, N) / Ritz values, HMAT(cnt, cnt) / VJ(N, cnt)."""
    n = vj.shape[0]
    save_records(path, [struct.pack("<ii", int(cnt), int(n)),
                        np.ascontiguousarray(ritz[:cnt], dtype="<f8").tobytes()
                        + np.asfortranarray(hmat[:cnt, :cnt], dtype="<f8").tobytes(order="F"),
                        np.asfortranarray(vj[:, :cnt], dtype="<f8").tobytes(order="F")])


def load_pist_basis(path):
    r = load_records(path)
    cnt, n = struct.unpack("<ii", r[0][:8])
    a = np.frombuffer(r[1], dtype="<f8")
    ritz = a[:cnt].copy()
    hmat = a[cnt:cnt + cnt * cnt].reshape(cnt, cnt, order="F").copy()
    vj = np.frombuffer(r[2], dtype="<f8").reshape(n, cnt, order="F").copy()
    return cnt, ritz, hmat, vj


def save_hw(path, hw, binary: bool = True) -> None:
    """The HW file of the OSBW window (saveHW, src/iterate/module/osb.io.h:297-319):
    unformatted sequential records (count) / HW(count, count), or with
    ``binary=False`` the list-directed text form (count, then HW column by
    column)."""
    hw = np.asarray(hw, dtype=np.float64)
    cnt = hw.shape[0]
    if hw.shape != (cnt, cnt):
        raise ValueError("HW must be square")
    if binary:
        save_records(path, [struct.pack("<i", cnt), np.asfortranarray(hw, dtype="<f8").tobytes(order="F")])
        return
    with open(path, "w") as f:
        f.write(f" {cnt}\n")
        flat = hw.ravel(order="F")
        for i in range(0, flat.size, 3):
            f.write(" " + " ".join(repr(float(v)) for v in flat[i:i + 3]) + "\n")


def load_hw(path, count: int, binary: bool = True) -> np.ndarray:
    """loadHW (osb.io.h:240-264): the HW file of a window of ``count`` states;
    ValueError when the file holds another count (loadHW returns .false.).
    The text form accepts Fortran list-directed repeats (``r*value``)."""
    if binary:
        r = load_records(path)
        if len(r) < 2 or len(r[0]) < 4:
            raise ValueError(f"{path}: not an HW file")
        cnt = struct.unpack("<i", r[0][:4])[0]
        if cnt != count:
            raise ValueError(f"{path}: window of {cnt} states, expected {count}")
        a = np.frombuffer(r[1], dtype="<f8")
        if a.size != cnt * cnt:
            raise ValueError(f"{path}: truncated HW")
        return a.reshape(cnt, cnt, order="F").copy()
    with open(path) as f:
        toks = f.read().replace(",", " ").split()
    vals = []
    for t in toks:
        if "*" in t:
            rep, v = t.split("*", 1)
            vals.extend([_real(v)] * int(rep))
        else:
            vals.append(_real(t))
    if not vals or int(vals[0]) != count:
        raise ValueError(f"{path}: window of {int(vals[0]) if vals else 0} states, expected {count}")
    a = np.array(vals[1:1 + count * count], dtype=np.float64)
    if a.size != count * count:
        raise ValueError(f"{path}: truncated HW")
    return a.reshape(count, count, order="F")


def load_data(path, n: int) -> np.ndarray:
    """Read the first ``n`` doubles of an unformatted sequential record."""
    out = bytearray()
    with open(path, "rb") as f:
        while True:
            hdr = f.read(4)
            if len(hdr) != 4:
                raise ValueError(f"{path}: truncated record marker")
            lead = struct.unpack("<i", hdr)[0]
            size = abs(lead)
            chunk = f.read(size)
            if len(chunk) != size:
                raise ValueError(f"{path}: truncated record")
            out += chunk
            tail = f.read(4)
            if len(tail) != 4:
                raise ValueError(f"{path}: truncated trailing marker")
            if lead >= 0:
                break
    if len(out) < 8 * n:
        raise ValueError(f"{path}: record holds {len(out) // 8} doubles, need {n}")
    return np.frombuffer(bytes(out[:8 * n]), dtype="<f8").astype(np.float64)


def save_data_dir(path, data: np.ndarray) -> None:
    """Direct-access record of raw doubles (``saveDataDir``)."""
    np.ascontiguousarray(data, dtype="<f8").tofile(path)


def load_data_dir(path, n: int) -> np.ndarray:
    """Read ``n`` raw doubles (``loadDataDir``)."""
    a = np.fromfile(path, dtype="<f8", count=n)
    if a.size != n:
        raise ValueError(f"{path}: holds {a.size} doubles, need {n}")
    return a.astype(np.float64)


def write_problem_files(problem, directory, inp: OSBInput | None = None) -> OSBInput:
    """Write H0/RES/DEP of a generated problem plus a matching parameter file."""
    import os
    os.makedirs(directory, exist_ok=True)
    inp = inp or OSBInput()
    inp = dataclasses.replace(inp, sF=3, sN=tuple(problem.sizes), sDEP=tuple(problem.dep),
                              H0File=os.path.join(directory, "H0.dat"),
                              RESFile=os.path.join(directory, "RES.dat"),
                              DEPFile=os.path.join(directory, "DEP.dat"))
    save_data(inp.H0File, problem.H0)
    save_data_dir(inp.RESFile, problem.RES)
    save_data_dir(inp.DEPFile, problem.DEP)
    with open(os.path.join(directory, "input.txt"), "w") as f:
        f.write(write_input(inp))
    return inp
