"""Host-side mirror of the reference's OSB module and iterate driver.

The serial driver ``prog_diag`` (src/iterate/prog/osb.drv.f90:3-38) and its MPI
twin (posb2.drv.f90:5-44) do: read the stdin parameter file (myReadOSB), size
the module (calOSB), load H0/RES/DEP (loadInitData), build the preconditioner
(progDiag -> myDiag) and run PIST (progPistEig -> OSB_PISTCONV).  :class:`OSB`
keeps the same steps and names; every numerical step runs on the GPU through
the C ABI (``scalit_gb300.capi``).

    python -m scalit_gb300.osb < input.txt
"""
from __future__ import annotations

import sys
import time

import numpy as np

from . import capi, refio


class OSB:
    """Module state: the parameter record plus the device context."""

    def __init__(self, inp: refio.OSBInput, device: int = 0, precision: int = capi.PREC_FP64):
        self.inp = inp
        self.device = device
        self.precision = precision
        self.ctx = None
        self.stats = None

    # readOSB (osb.print.h:2, 192-246)
    @classmethod
    def read(cls, text: str, **kw) -> "OSB":
        return cls(refio.read_input(text), **kw)

    # loadInitData (osb.io.h:2-42)
    def load_init_data(self) -> bool:
        inp = self.inp
        # sCX (loadH0 / loadDEP / loadOutH, osb.io.h:46-54,211-238): H0, DEP and
        # OUTH are COMPLEX*16 records of the same lengths (loadData_CX,
        # loadDataDir_CX); RES stays real
        def cxv(a):
            return a.view(np.complex128)
        mult = 2 if inp.sCX else 1
        H0 = refio.load_data(inp.H0File, mult * inp.h0_len)
        OUTH = None
        if inp.sNDVR:
            OUTH = refio.load_data_dir(inp.OUTHFile, mult * inp.sN[inp.sF - 1] * inp.my_len)
            RES = np.zeros(inp.my_len)
        else:
            RES = refio.load_data_dir(inp.RESFile, inp.my_len)
        DEP = refio.load_data_dir(inp.DEPFile, mult * inp.dep_len) if inp.dep_len else None
        self.ctx = capi.Context(inp.sN[:inp.sF], inp.sDEP[:inp.sF], ndvr=inp.sNDVR, device=self.device)
        if inp.sCX:
            self.ctx.load_cx(cxv(H0), RES, None if DEP is None else cxv(DEP), None if OUTH is None else cxv(OUTH))
        else:
            self.ctx.load(H0, RES, DEP, OUTH)
        # absorbing potentials (osb.io.h:18-30): APP for the resonance jobs, APP and APR for CRP
        if inp.sJOB in (refio.JOB_RES1, refio.JOB_RES2):
            self.ctx.set_absorbing(refio.load_data_dir(inp.APPFile, inp.my_len))
        elif inp.sJOB in (refio.JOB_CRP, refio.JOB_CRP1, refio.JOB_CRP2):
            self.ctx.set_absorbing(refio.load_data_dir(inp.APPFile, inp.my_len),
                                   refio.load_data_dir(inp.APRFile, inp.my_len))
        self.ctx.set_shift(inp.sOSBW[0])
        self.ctx.set_precond(inp.sOSB if inp.sOSB in (1, 2, 3) else 1, inp.sOSBW[1], inp.sOSBW[2])
        return True

    # progDiag (osb.progDiag.h:6-51): build, or load a saved preconditioner (sVOSB < 0)
    def prog_diag(self, log=print):
        inp = self.inp
        t0 = time.perf_counter()
        if inp.sVOSB < 0:
            V = refio.load_data_dir(inp.VOSBFile, self.ctx.vosb_len)
            E = refio.load_data_dir(inp.EigFile, inp.my_len)
            self.ctx.set_osb(V, E)
        else:
            self.stats = self.ctx.build_osb(inp.sBJ[0], inp.sBJ[1])
            if log:
                for l in range(inp.sF - 1, -1, -1):
                    eff = self.stats[l]
                    blk = inp.my_blk[l]
                    log(f"  BJ Diag.: Level:{l + 1:4d}.   Grid Size:{inp.sN[l]:6d}   # of Blocks:{blk:6d}")
                    log(f" Aver. # of Sweeps:{eff[4] / blk:10.5f}.    Aver. OffDiag/Diag:{eff[2] / eff[4]:10.6f}")
                    log(f" Jacobi Effi: Min:{eff[0]:10.5f},   Max:{eff[1]:10.5f},  Mean:{eff[2] / blk:10.5f}")
            if inp.sVOSB > 0:
                V, E = self.ctx.get_osb()
                refio.save_data_dir(inp.VOSBFile, V)
                refio.save_data_dir(inp.EigFile, E)
        if log:
            log(f" Time for block diagonalization (s): {time.perf_counter() - t0:.3f}")
        if inp.sOSB == refio.TOSBW:
            self.init_osbw(log)

    # initOSBW (osb.osbw.h:2-50), bound-state job: sHW >= 0 forms the window
    # matrix (sHW > 0 also writes it, saveHW), sHW < 0 reads it (loadHW)
    def init_osbw(self, log=print):
        inp = self.inp
        mE0, mDE, mBeta, mCnt = inp.sOSBW
        t0 = time.perf_counter()
        if log:
            log(f" original window width: {mDE}  size: {mCnt}")
        if inp.sHW >= 0:
            _, de = self.ctx.build_osbw(mE0, mCnt, mDE, capi.TA1)
            if inp.sHW > 0:
                _, HW = self.ctx.get_osbw()
                refio.save_hw(inp.HWFile, HW)
        else:
            de = self.ctx.set_osbw(mE0, mCnt, mDE, refio.load_hw(inp.HWFile, mCnt), capi.TA1)
        inp.sOSBW = (mE0, de, mBeta, mCnt)             # adjustWinSize updates sOSBW%mDE
        if log:
            log(f" final window width: {de}  window size: {mCnt}")
            log(f" Time to calculate Hij for Energy Window: {time.perf_counter() - t0:.3f}")

    # OSB_PISTCONV (osbw.pistconv.h:16-50) with setPISTConvParam (:303-333)
    def pist(self, x0=None, seed=0, verbose=False, basis=False):
        inp = self.inp
        mE0, mTol, mStart, mStep, mMax, mNum, mGap = inp.sConv
        if x0 is None:
            x0 = np.random.default_rng(seed).random(inp.my_len)   # random_number(X)
        return self.ctx.pist(x0, mNum, mE0, mTol, startcnt=mStart, stepcnt=mStep, m_max=mMax,
                             gap=mGap, qmr_max=inp.sQMR[0], qmr_tol=inp.sQMR[1], qmr_ntype=-1,
                             precision=self.precision, ntype=0, verbose=verbose, basis=basis)

    # setPISTConvParam (osbw.pistconv.h:303-333)
    def pist_params(self):
        mE0, mTol, mStart, mStep, mMax, mNum, mGap = self.inp.sConv
        start = 2 * mNum if mStart < mNum else mStart
        return dict(e0=mE0, etol=mTol, startcnt=start, stepcnt=5 if mStep < 1 else mStep,
                    stepeig=1 if mGap < 1 else mGap, m_max=start + mNum if mMax < start else mMax)

    # OSB_PISTCONVDX1 / OSB_PISTCONVDX2 (osbw.pistconv.h:102-143, 204-245):
    # resonances of H - i AP by the symmetric (JOB_RES1) or the conjugate
    # (JOB_RES2) complex PIST; QMR_CX on (H - E0 - i AP) with the
    # preconditioner's absorbing term when sAP is set
    def pist_resonances(self, x0=None, seed=0):
        inp = self.inp
        prm = self.pist_params()
        if x0 is None:
            rng = np.random.default_rng(seed)                     # randMat_CX
            x0 = rng.random(inp.my_len) + 1j * rng.random(inp.my_len)
        return self.ctx.pist_cx(x0, inp.sConv[5], prm["e0"], prm["etol"], prm["m_max"],
                                startcnt=prm["startcnt"], stepcnt=prm["stepcnt"], stepeig=prm["stepeig"],
                                h0_ntype=capi.TMAP0, ls_ntype=capi.TMAP,
                                ls_px_ntype=capi.TMAP if inp.sAP else capi.TA1, conv=-1,
                                qmrmax=inp.sQMR[0], qmrtol=inp.sQMR[1],
                                conjugate=inp.sJOB == refio.JOB_RES2)

    # the CRP job of progPistEig (osbw.progEig.h:55-63): N(E) at
    # E = mE0 + (i - 1) mTol, i = 1..mNum, with mGap Lanczos steps
    def crp_energies(self):
        mE0, mTol, _, _, _, mNum, _ = self.inp.sConv
        return mE0 + mTol * np.arange(mNum)

    def crp(self, seed=0):
        inp = self.inp
        energies = self.crp_energies()
        return energies, self.ctx.crp(energies, inp.sConv[6], qmrmax=inp.sQMR[0], qmrtol=inp.sQMR[1], conv=-1,
                                      sap=inp.sAP, seed=seed)

    # progPistEig (osbw.progEig.h:6-98)
    def prog_pist_eig(self, log=print, **kw):
        t0 = time.perf_counter()
        if log:
            log(" ================================================")
            log("      Get  Eigen Values Using PIST method        ")
            log(" ================================================")
        job = self.inp.sJOB
        if job in (refio.JOB_CRP, refio.JOB_CRP1, refio.JOB_CRP2):
            if log:
                log(" ------  CRP calculation for Real Version of H0  -------")
            energies, crp = self.crp()
            if log:
                for i, (e, v) in enumerate(zip(energies, crp), 1):
                    log(f"Step:{i:5d} | Energy:{e:10.6f} | CRP:{v:15.9f}")
                log(f" Time to get PIST Eigen values:(sec) {time.perf_counter() - t0:.3f}")
            return len(crp), crp, 0.0, {"energies": energies}
        if job in (refio.JOB_RES1, refio.JOB_RES2):
            if log:
                log(" ------  Resonance states for Real Version of H0  -------")
                log(" ------ Using Symmetric version of PIST  -------" if job == refio.JOB_RES1 else
                    " ------ Using Conjugate version of PIST  -------")
            st, eig, res = self.pist_resonances()
            if log:
                log(f" Max Lanczos Error: {res:.15E}  Eigen Values:")
                for e in eig:
                    log(f"{e.real:25.15E}  {e.imag:25.15E}")
                log(f" Time to get PIST Eigen values:(sec) {time.perf_counter() - t0:.3f}")
            return st, eig, res, {}
        if log:
            log(" ------  Bound states for Real Version of H0  -------")
        if self.inp.sPT != 0:
            kw = dict(kw, basis=True)
        st, eig, res, info = self.pist(**kw)
        if self.inp.sPT != 0 and st > 0:
            refio.save_pist_basis(self.inp.PTFile, info["cnt"], info["ritz"], info["hmat"], info["vj"])
            if log:
                log(f" PIST basis and HMAT written to {self.inp.PTFile}")
        if log:
            log(f" Max Lanczos Error: {res:.15E}  Eigen Values:")
            for i in range(0, len(eig), 3):
                log("  ".join(f"{e:25.15E}" for e in eig[i:i + 3]))
            log(f" Time to get PIST Eigen values:(sec) {time.perf_counter() - t0:.3f}")
        return st, eig, res, info

    def close(self):
        if self.ctx is not None:
            self.ctx.close()
            self.ctx = None


def main(argv=None):
    text = sys.stdin.read()
    osb = OSB.read(text)
    capi.load(build_if_missing=True)
    if not osb.load_init_data():
        print(" Error in loading data", file=sys.stderr)
        return 1
    osb.prog_diag()
    st, eig, res, info = osb.prog_pist_eig(verbose=True)
    osb.close()
    return 0 if st > 0 else 2


if __name__ == "__main__":
    sys.exit(main())
