"""Input formats of the iterate stage and the synthetic generator (no GPU)."""
import numpy as np
import pytest

from scalit_gb300 import hamiltonian as hm
from scalit_gb300 import refio


def test_input_roundtrip(tmp_path):
    inp = refio.OSBInput(sN=(24, 32, 20), sBJ=(15, 1e-5), sQMR=(300, 1e-4),
                         sConv=(0.001, 1e-9, 40, 5, 400, 20, 1), sOSBW=(0.0, 0.002, 0.0, 0))
    text = refio.write_input(inp)
    back = refio.read_input(text)
    for k in ("sF", "sN", "sDEP", "sJOB", "sOSB", "sBJ", "sQMR", "sConv", "sOSBW", "H0File",
              "RESFile", "DEPFile"):
        assert getattr(back, k) == getattr(inp, k), k


def test_input_fortran_spellings():
    text = """3 24 32 20
 .false. .FALSE. .true.
 1, 1
 F F F F
 20 1.0D-4 300 1.0d-4
 0.0D0 1D-8 0 5 0 20 1
 0.0 -0.002 0.0 0
 0 0 0 0 0
H0.dat
RES.dat
DEP.dat
"""
    inp = refio.read_input(text)
    assert inp.sN == (24, 32, 20)
    assert inp.sDEP == (False, False, True)
    assert inp.sBJ == (20, 1e-4)
    assert inp.sOSBW[1] == 0.002          # |mDE| (osb.print.h:212)
    assert inp.DEPFile == "DEP.dat"


def test_dep1_forced_false():
    text = "2 4 5\nT T\n1 1\nF F F F\n1 0.1 1 0.1\n0 0 0 0 0 1 0\n0 0 0 0\n0 0 0 0 0\nH0\nRES\nDEP\n"
    assert refio.read_input(text).sDEP == (False, True)


def test_sequential_record_roundtrip(tmp_path):
    a = np.random.default_rng(0).standard_normal(1000)
    path = tmp_path / "H0.dat"
    refio.save_data(path, a)
    raw = path.read_bytes()
    assert int.from_bytes(raw[:4], "little") == 8000 == int.from_bytes(raw[-4:], "little")
    np.testing.assert_array_equal(refio.load_data(path, 1000), a)
    with pytest.raises(ValueError):
        refio.load_data(path, 1001)


def test_direct_access_roundtrip(tmp_path):
    a = np.random.default_rng(1).standard_normal(77)
    path = tmp_path / "RES.dat"
    refio.save_data_dir(path, a)
    assert path.stat().st_size == 77 * 8
    np.testing.assert_array_equal(refio.load_data_dir(path, 77), a)


def test_truncated_file_rejected(tmp_path):
    path = tmp_path / "bad.dat"
    path.write_bytes(b"\x10\x00\x00\x00" + b"\x00" * 8)
    with pytest.raises(ValueError):
        refio.load_data(path, 2)


def test_sizes_follow_calosb():
    inp = refio.OSBInput(sF=3, sN=(24, 32, 20))
    assert inp.my_dim == (1, 24, 768)
    assert inp.my_blk == (640, 20, 1)
    assert inp.my_len == 15360
    assert inp.h0_len == 24 ** 2 + 32 ** 2 + 20 ** 2
    assert inp.dep_len == 768


def test_sine_dvr_closed_form():
    _, T = hm.sine_dvr(17, 1.5, 4.0, 14582.6)
    np.testing.assert_allclose(T, hm.sine_dvr_closed_form(17, 1.5, 4.0, 14582.6), atol=1e-16)


def test_legendre_dvr():
    x, w, T, K = hm.legendre_dvr(12)
    np.testing.assert_allclose(T.T @ T, np.eye(12), atol=1e-13)
    ev = np.sort(np.linalg.eigvalsh(K))
    np.testing.assert_allclose(ev, [j * (j + 1) for j in range(12)], atol=1e-9)


def test_potential_gradient_fd():
    pes = hm.PES(amp1=0.001, amp3=0.0005, width1=1.3, width3=0.8)
    r = np.linspace(1.6, 3.9, 5)[:, None, None]
    R = np.linspace(2.5, 7.5, 4)[None, :, None]
    c = np.linspace(-0.9, 0.9, 3)[None, None, :]
    g = hm.potential_grad(r, R, c, pes)
    p0 = pes.params()
    for k in range(12):
        h = 1e-6 * max(abs(p0[k]), 1.0)
        pp, pm = p0.copy(), p0.copy()
        pp[k] += h
        pm[k] -= h
        fd = (hm.potential(r, R, c, pes.with_params(pp)) - hm.potential(r, R, c, pes.with_params(pm))) / (2 * h)
        np.testing.assert_allclose(g[k], fd, rtol=1e-5, atol=1e-10)


def test_problem_files(tmp_path):
    p = hm.build_problem(hm.Grid3(4, 5, 3), hm.PES())
    inp = refio.write_problem_files(p, tmp_path)
    back = refio.read_input((tmp_path / "input.txt").read_text())
    np.testing.assert_array_equal(refio.load_data(back.H0File, back.h0_len), p.H0)
    np.testing.assert_array_equal(refio.load_data_dir(back.RESFile, back.my_len), p.RES)
    np.testing.assert_array_equal(refio.load_data_dir(back.DEPFile, back.dep_len), p.DEP)


def test_records_and_subrecords(tmp_path, monkeypatch):
    recs = [b"\x01\x02\x03\x04" * 5, b"", b"x" * 37]
    path = tmp_path / "r.dat"
    monkeypatch.setattr(refio, "_MAX_SUBRECORD", 8)       # force sub-records
    refio.save_records(path, recs)
    assert refio.load_records(path) == recs


def test_pist_basis_file_roundtrip(tmp_path):
    rng = np.random.default_rng(3)
    cnt, n = 5, 11
    ritz = rng.standard_normal(cnt)
    hmat = rng.standard_normal((cnt, cnt))
    vj = rng.standard_normal((n, cnt))
    path = tmp_path / "PT.dat"
    refio.save_pist_basis(path, cnt, ritz, hmat, vj)
    raw = path.read_bytes()
    assert int.from_bytes(raw[:4], "little") == 8                       # record 1: (cnt, N)
    assert int.from_bytes(raw[4:8], "little") == cnt
    c2, r2, h2, v2 = refio.load_pist_basis(path)
    assert c2 == cnt
    np.testing.assert_array_equal(r2, ritz)
    np.testing.assert_array_equal(h2, hmat)
    np.testing.assert_array_equal(v2, vj)


def test_hw_file_roundtrip(tmp_path):
    """saveHW / loadHW (osb.io.h:240-319), both forms; a file of another window size is refused."""
    rng = np.random.default_rng(4)
    a = rng.standard_normal((6, 6))
    hw = (a + a.T) / 2
    for binary in (True, False):
        path = tmp_path / f"hw_{binary}.dat"
        refio.save_hw(path, hw, binary=binary)
        np.testing.assert_array_equal(refio.load_hw(path, 6, binary=binary), hw)
        with pytest.raises(ValueError):
            refio.load_hw(path, 5, binary=binary)
    raw = (tmp_path / "hw_True.dat").read_bytes()
    assert int.from_bytes(raw[:4], "little") == 4 and int.from_bytes(raw[4:8], "little") == 6
    txt = tmp_path / "hw_rep.txt"                       # list-directed repeats: r*value, D exponents
    txt.write_text(" 2\n 2*1.5D0 0.25\n -3.0\n")
    np.testing.assert_array_equal(refio.load_hw(txt, 2, binary=False), [[1.5, 0.25], [1.5, -3.0]])


@pytest.mark.parametrize("job,names", [(2, ("APP.dat",)), (3, ("APP.dat",)), (4, ("APP.dat", "APR.dat")),
                                       (6, ("APP.dat", "APR.dat"))])
def test_input_absorbing_potential_files(job, names):
    """myReadOSB (osb.print.h:230-234): the resonance jobs name APPFile, the CRP
    jobs APPFile and APRFile, after the DEP file and before the optional files."""
    inp = refio.OSBInput(sJOB=job, sAP=True, sVOSB=1, VOSBFile="V.dat", EigFile="E.dat",
                         APPFile=names[0], APRFile=names[1] if len(names) > 1 else "")
    text = refio.write_input(inp)
    lines = text.splitlines()
    i = lines.index("DEP.dat")
    assert tuple(lines[i + 1:i + 1 + len(names)]) == names
    assert lines[i + 1 + len(names)] == "V.dat"
    back = refio.read_input(text)
    assert back.sJOB == job and back.sAP
    assert back.APPFile == "APP.dat" and back.APRFile == (names[1] if len(names) > 1 else "")
    assert back.VOSBFile == "V.dat" and back.EigFile == "E.dat"


def test_driver_parameters_without_a_device():
    """setPISTConvParam (osbw.pistconv.h:303-333) and the CRP job's energy grid
    (osbw.progEig.h:55-63) as the driver derives them."""
    from scalit_gb300 import osb
    o = osb.OSB(refio.OSBInput(sJOB=refio.JOB_CRP, sConv=(0.5, 0.01, 0, 0, 0, 4, 9)))
    np.testing.assert_allclose(o.crp_energies(), [0.5, 0.51, 0.52, 0.53])
    assert o.pist_params() == dict(e0=0.5, etol=0.01, startcnt=8, stepcnt=5, stepeig=9, m_max=12)
    o2 = osb.OSB(refio.OSBInput(sConv=(0.1, 1e-8, 30, 7, 100, 20, 0)))
    assert o2.pist_params() == dict(e0=0.1, etol=1e-8, startcnt=30, stepcnt=7, stepeig=1, m_max=100)
    o2.close()
    o.close()
