"""Shared case builders: one configuration drives both the CUDA engine (through
``dasp_gb300.centcmod``) and the oracle, on identical inputs."""
from __future__ import annotations

import numpy as np

from dasp_gb300.screens import gaussian_psf, lgs_psfs, von_karman_screen
from dasp_gb300.tel import Pupil

DEFAULTS = dict(nthreads=4, readnoise=0.0, readbg=0.0, addPoisson=0, noiseFloor=0.0, sig=1e4,
                skybrightness=0.0, calsource=0, pxlPower=1.0, nintegrations=1, nlatency=0, seed=7,
                minarea=0.5, opticalBinning=0, centWeight=None, correlationCentroiding=0, corrThresh=0.0,
                corrPattern=None, corrimg=None, threshType=0, imageOnly=0, useBrightest=0,
                preBinningFactor=1, parabolicFit=0, gaussianFitVals=None)


class Case:
    """A WFS configuration plus its inputs."""

    def __init__(self, nsubx=8, p=8, N=16, C=None, m=None, ncen=None, obs=0.25, psf=None, phase_seed=0,
                 r0=0.15, L0=30.0, Dtel=4.2, wavelength=640.0, amp=False, **kw):
        self.nsubx, self.p, self.N = nsubx, p, N
        self.C = N if C is None else C
        self.m = self.C // 2 if m is None else m
        self.ncen = self.m if ncen is None else ncen
        npup = nsubx * p
        self.pup = Pupil(npup, npup / 2.0, npup / 2.0 * obs)
        self.params = dict(DEFAULTS)
        self.params.update(kw)
        self.nsubaps = nsubx * nsubx
        self.W = npup
        self.phase_args = (npup, Dtel, r0, L0, phase_seed, wavelength)
        phs = von_karman_screen(npup, Dtel, r0, L0, phase_seed, wavelength)
        if amp:
            a = 1.0 + 0.2 * np.random.default_rng(phase_seed + 99).standard_normal((npup, npup))
            phs = np.ascontiguousarray(np.stack([phs, np.abs(a).astype(np.float32)]), dtype=np.float32)
        self.phs = np.ascontiguousarray(phs, dtype=np.float32)
        if isinstance(psf, np.ndarray):
            self.psf = psf
        elif psf == "gauss":
            self.psf = gaussian_psf(self.P_default(), 1.5)
        elif psf == "gauss4d":
            frac = self.pup.getSubarea(nsubx) / (p * p)
            self.psf = lgs_psfs(nsubx, self.P_default(), 1.2, 6.0, subap_area=frac)
        else:
            self.psf = None

    def P_default(self):
        return self.params.pop("psfsize", None) or self.C

    def new_phase(self, seed):
        npup, Dtel, r0, L0, _, wl = self.phase_args
        ph = von_karman_screen(npup, Dtel, r0, L0, seed, wl)
        if self.phs.ndim == 3:
            out = self.phs.copy()
            out[0] = ph
            return out
        return ph

    # -- engine --
    def engine(self, phs=None, cents=None, bimg=None, inputImage=None, subapLocation=None, no_phase=False):
        from dasp_gb300.centcmod import centcmod
        p = self.params
        self.cents = np.zeros((self.nsubaps * 2,), np.float32) if cents is None else cents
        self.bimg = np.zeros((self.nsubx, self.nsubx, self.m, self.m), np.float32) if bimg is None else bimg
        return centcmod(p["nthreads"], self.nsubx, self.ncen, self.N, self.C, self.m, self.p, p["readnoise"],
                        p["readbg"], p["addPoisson"], p["noiseFloor"], p["sig"], p["skybrightness"],
                        p["calsource"], p["pxlPower"], p["nintegrations"], p["nlatency"], p["seed"],
                        None if no_phase else (self.phs if phs is None else phs), self.pup, self.psf, self.cents,
                        self.bimg, p["minarea"], p["opticalBinning"], p["centWeight"], p["correlationCentroiding"],
                        p["corrThresh"], p["corrPattern"], p["corrimg"], p["threshType"], p["imageOnly"],
                        p["useBrightest"], p["preBinningFactor"], p["parabolicFit"], p["gaussianFitVals"],
                        inputImage, subapLocation)

    # -- the reference's own module (oracle/_ref) --
    def reference(self, phs=None, cents=None, bimg=None, inputImage=None, subapLocation=None, **over):
        """The reference's cent module on this case's inputs.  Its outputs land
        in ``self.ref_cents`` / ``self.ref_bimg`` (or the arrays given);
        ``over`` replaces parameters for this handle only."""
        from oracle.ref_cent import RefCent
        p = dict(self.params)
        p.update(over)
        self.ref_phs = np.ascontiguousarray(self.phs if phs is None else phs, dtype=np.float32)
        self.ref_cents = np.zeros((self.nsubaps * 2,), np.float32) if cents is None else cents
        self.ref_bimg = np.zeros((self.nsubx, self.nsubx, self.m, self.m), np.float32) if bimg is None else bimg
        psf = None if self.psf is None else np.ascontiguousarray(self.psf, dtype=np.float32)
        return RefCent(p["nthreads"], self.nsubx, self.ncen, self.N, self.C, self.m, self.p, p["readnoise"],
                       p["readbg"], p["addPoisson"], p["noiseFloor"], p["sig"], p["skybrightness"],
                       p["calsource"], p["pxlPower"], p["nintegrations"], p["nlatency"], p["seed"],
                       self.ref_phs, self.pup, psf, self.ref_cents, self.ref_bimg, p["minarea"],
                       p["opticalBinning"], p["centWeight"], p["correlationCentroiding"], p["corrThresh"],
                       p["corrPattern"], p["corrimg"], p["threshType"], p["imageOnly"], p["useBrightest"],
                       p["preBinningFactor"], p["parabolicFit"], p["gaussianFitVals"], inputImage, subapLocation)

    # -- oracle --
    def oracle(self, mode="f32"):
        from oracle.shwfs_oracle import CentOracle
        p = self.params
        gf = p["gaussianFitVals"]
        return CentOracle(nsubx=self.nsubx, phasesize=self.p, fftsize=self.N, clipsize=self.C, nimg=self.m,
                          ncen=self.ncen, pupfn=self.pup.perSubap(self.nsubx, 0),
                          subflag=self.pup.getSubapFlag(self.nsubx, p["minarea"]),
                          fracSubArea=(self.pup.getSubarea(self.nsubx) / (self.p * self.p)).astype(np.float32),
                          sig=p["sig"], readnoise=p["readnoise"], readbg=p["readbg"], addPoisson=p["addPoisson"],
                          noiseFloor=p["noiseFloor"], skybrightness=p["skybrightness"], calsource=p["calsource"],
                          pxlPower=p["pxlPower"], nintegrations=p["nintegrations"], nlatency=p["nlatency"],
                          seed=p["seed"], nthreads=p["nthreads"], spotpsf=self.psf,
                          opticalBinning=p["opticalBinning"], centWeight=p["centWeight"],
                          threshType=p["threshType"], imageOnly=p["imageOnly"], useBrightest=p["useBrightest"],
                          preBinningFactor=p["preBinningFactor"], parabolicFit=p["parabolicFit"],
                          gaussianFit=0 if gf is None else 1,
                          gaussianMinVal=0.0 if gf is None else gf[0],
                          gaussianReplaceVal=0.0 if gf is None else gf[1],
                          correlationCentroiding=p["correlationCentroiding"], corrThresh=p["corrThresh"],
                          corrPattern=p["corrPattern"], mode=mode)

    def oracle_run(self, orc, phs=None, cents=None, bimg=None):
        phs = self.phs if phs is None else phs
        cents = np.zeros((self.nsubaps * 2,), np.float32) if cents is None else cents
        bimg = np.zeros((self.nsubaps, self.m, self.m), np.float32) if bimg is None else bimg
        if phs.ndim == 3:
            orc.run(phs[0], cents, bimg, amp=phs[1])
        else:
            orc.run(phs, cents, bimg)
        return cents, bimg

    def lit(self):
        return self.pup.getSubapFlag(self.nsubx, self.params["minarea"]).reshape(-1) == 1
