"""Generates the golden fixtures in this directory from the reference itself.

Runs the reference's own FP64 CPU path (oracle/_ref/libscref.so, built from
the reference sources by oracle/build_ref.sh) on small synthetic cases and
stores, per case: the parameters, the image, the prepared coefficient arrays
and switch points (known answers for the host preparation), and for fit cases
the chi^2 sums. Usage (needs the reference sources and the built oracle/_ref):

    python tests/golden/make_golden.py

Each case also stores "cond", the per-pixel sensitivity of the reference's
result to one-ulp differences of the math library (oracle.cpu_oracle.condition,
measured with the reference-pinned oracle, or, for the generic pixel function
that the oracle does not restate, oracle.refbind.condition on the reference's
own probe build): pixels where the reference's own
result moves by more than 1e-12 under such perturbations cannot be reproduced
to 1e-10 by another math library and are compared against that envelope.

The cases are the benchmark workloads on coarser grids with the same q-range
(crystalscatter_gb300.configs.scaled) plus variants that reach other branches
(quadrant mirroring, midpoint geometry, beam offset, core/shell spheres,
cylinder orientations, BCT parameter sets) and rejected parameter sets.
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from crystalscatter_gb300 import configs as C  # noqa: E402
from oracle import cpu_oracle, refbind  # noqa: E402

ARRAYS = ["carr1p", "carr2p", "carr3p", "carr4p", "carr5p", "carr6p", "carr1f", "carr2f", "carr4f", "carr5f",
          "carr6f", "carr11pm"]
SCALARS = ["limq1", "limq2", "limq3", "limq4", "limq5", "limq6", "limq1f", "limq4f", "norm", "order", "orcase",
           "peakmax1", "peakmax2", "latpar1", "latpar2", "latpar3", "newswitch"]


def image_cases():
    cases = {
        "sphere_g64": C.scaled(C.SPHERE, 64),
        "cyl_gauss_g32": C.scaled(C.CYL_GAUSS, 32),
        "cyl_gauss_x_g24": C.scaled(C.CYL_GAUSS_X, 24),
        "sphere_fcc_g32": C.scaled(C.SPHERE_FCC, 32),
        "sphere_fcc_hkl3_g24": dict(C.scaled(C.SPHERE_FCC, 24), HKLmax=3),
        # quadrant mirroring and geometry variants
        "sphere_q1_expand_g32": dict(C.scaled(C.SPHERE, 32), RadioButtonQ1=1, RadioButtonQ4=0, ExpandImage=1),
        "sphere_q2_expand_g32": dict(C.scaled(C.SPHERE, 32), RadioButtonQ2=1, RadioButtonQ4=0, ExpandImage=1),
        "sphere_q1_noexpand_g32": dict(C.scaled(C.SPHERE, 32), RadioButtonQ1=1, RadioButtonQ4=0, ExpandImage=0),
        "sphere_midpoint_g32": dict(C.scaled(C.SPHERE, 32), CenterBeam=0, EditQmax=2.0),
        "sphere_beamoffset_g32": dict(C.scaled(C.SPHERE, 32), BeamPosX=5.5, BeamPosY=-3.0),
        "sphere_bgiso_g32": dict(C.scaled(C.SPHERE, 32), Base=1e-3, iso=0.25, ifluc=0.1, rfluc=2.0, I0=7.5),
        "sphere_coreshell_g32": dict(C.scaled(C.SPHERE, 32), ComboBoxInterior=1, EditRadiusi=14.0, EditRho=0.3),
        "sphere_wide_sigma_g32": dict(C.scaled(C.SPHERE, 32), EditSigma=0.3),
        # cylinder orientations, no lattice
        "cyl_gauss_y_g24": dict(C.scaled(C.CYL_GAUSS, 24), phi=90.0),
        "cyl_gauss_z_g24": dict(C.scaled(C.CYL_GAUSS, 24), theta=0.0, phi=0.0),
        "cyl_zdir_x_g32": dict(C.scaled(C.CYL_GAUSS, 32), Ordis=6, phi=0.0),
        "cyl_zdir_y_g32": dict(C.scaled(C.CYL_GAUSS, 32), Ordis=6, phi=90.0),
        "cyl_zdir_z_g32": dict(C.scaled(C.CYL_GAUSS, 32), Ordis=6, theta=0.0, phi=0.0),
        "cyl_zdir_gen_g32": dict(C.scaled(C.CYL_GAUSS, 32), Ordis=6, theta=60.0, phi=30.0),
    }
    for k in range(4):
        b = C.bct_set(k)
        cases[f"cyl_bct_set{k}_g24"] = C.scaled(b, 24)
    cases["cyl_bct_zaxis_g24"] = dict(C.scaled(C.bct_set(0), 24), theta=0.0, phi=0.0)
    # cube (its own pixel function) and the generic pixel function: other
    # lattices and peak shapes, cubes and cylinders on lattices, and the
    # specialised combinations with the new switch ignored
    sph = C.scaled(C.SPHERE_FCC, 24)
    cases["cube_g32"] = dict(C.scaled(C.SPHERE, 32), ComboBoxParticle=4)
    cases["cube_fcc_g24"] = dict(sph, ComboBoxParticle=4, Ordis=7)
    cases["sphere_bcc_g24"] = dict(sph, LType=4)
    cases["sphere_sc_g24"] = dict(sph, LType=7)
    cases["sphere_fcc_lorentz_g24"] = dict(sph, ComboBoxPeak=0)
    cases["sphere_fcc_modlor1_g24"] = dict(sph, ComboBoxPeak=2)
    cases["sphere_fcc_modlor2_g24"] = dict(sph, ComboBoxPeak=3)
    cases["sphere_fcc_voigt_g24"] = dict(sph, ComboBoxPeak=4, EditPeakPar=40.0)
    cases["sphere_fcc_pearson_g24"] = dict(sph, ComboBoxPeak=5, EditPeakPar=1.5)
    cases["sphere_fcc_twin_g24"] = dict(sph, LType=4, CheckBoxTwinned=1, EditCeff=0.7)
    # the anisotropic Gaussian peak: isotropic, perfect orientation (z
    # direction, and dbeta = 0), twinned; unit-cell axes and widths as set
    ani = dict(sph, ComboBoxPeak=7, EditAxis1x=1.0, EditAxis1y=0.2, EditAxis1z=0.0, EditAxis2x=0.0, EditAxis2y=1.0,
               EditAxis2z=0.1, EditAxis3x=0.0, EditAxis3y=0.0, EditAxis3z=1.0, Editdom1=60.0, Editdom2=45.0,
               Editdom3=30.0)
    cases["sphere_fcc_aniso_iso_g24"] = dict(ani, Ordis=7)
    cases["sphere_fcc_aniso_zdir_g24"] = dict(ani, Ordis=6)
    cases["sphere_fcc_aniso_dbeta0_g24"] = dict(ani, EditDbeta=0.0)
    cases["sphere_bcc_aniso_twin_g24"] = dict(ani, LType=4, Ordis=6, CheckBoxTwinned=1, EditCeff=0.7)
    cases["sphere_fcc_ignswitch_g24"] = dict(sph)
    cases["cyl_zdir_fcc_g24"] = dict(C.scaled(C.bct_set(2), 24), LType=5)
    cases["cyl_gauss_x_ignswitch_g16"] = C.scaled(C.CYL_GAUSS_X, 16)
    disk = dict(C.scaled(C.CYL_GAUSS, 32), ComboBoxParticle=2, Ordis=6, EditRadius=2.0, Length=30.0)
    cases["disk_zdir_x_g32"] = dict(disk, phi=0.0, theta=90.0)
    cases["disk_zdir_y_g32"] = dict(disk, phi=90.0, theta=90.0)
    cases["disk_zdir_z_iso_g32"] = dict(disk, phi=0.0, theta=0.0, iso=0.3)
    cases["disk_iso_g32"] = dict(disk, Ordis=7)
    # Gaussian orientation along an axis: the x axis switches from the triple
    # series to the delta/chi quadrature at 6 limq1, the y and z axes at
    # 6000 limq1; SigmaL 0.2 takes the quadrature's Ornstein-Zernike-like form
    dg24 = dict(C.scaled(C.CYL_GAUSS, 24), ComboBoxParticle=2, Ordis=0, EditRadius=2.0, Length=30.0)
    dg16 = dict(C.scaled(C.CYL_GAUSS, 16), ComboBoxParticle=2, Ordis=0, EditRadius=2.0, Length=30.0)
    cases["disk_gauss_x_g24"] = dict(dg24, phi=0.0, theta=90.0)
    cases["disk_gauss_x_oz_g16"] = dict(dg16, phi=0.0, theta=90.0, SigmaL=0.2)
    cases["disk_gauss_y_g24"] = dict(dg24, phi=90.0, theta=90.0)
    cases["disk_gauss_z_g24"] = dict(dg24, phi=0.0, theta=0.0, iso=0.2)
    cases["disk_gauss_z90_g16"] = dict(dg16, phi=90.0, theta=0.0)
    # disks on lattices: F(q) from the F coefficients
    dl = dict(sph, ComboBoxParticle=2, EditRadius=2.0, Length=12.0, SigmaL=0.1)
    cases["disk_iso_fcc_g24"] = dict(dl, Ordis=7)
    # (SigmaL 0.2: at 0.1 two pixels of this image move by 6e-9 under a
    # one-ulp change of sin or cos alone, which the probe's combined modes
    # do not show, so that no FP64 answer at 1e-10 exists for them)
    cases["disk_zdir_z_fcc_g24"] = dict(dl, Ordis=6, theta=0.0, phi=0.0, SigmaL=0.2)
    cases["disk_gauss_x_fcc_g24"] = dict(dl, Ordis=0, theta=90.0, phi=0.0, EditDbeta=15.0)
    cases["disk_zdir_y_bcc_g16"] = dict(C.scaled(C.SPHERE_FCC, 16), LType=4, ComboBoxParticle=2, EditRadius=2.0,
                                        Length=12.0, SigmaL=0.1, Ordis=6, theta=90.0, phi=90.0)
    # core/shell disks and z-direction cylinders (outer radius EditRadiusi,
    # relative contrast EditRho)
    dcs = dict(disk, ComboBoxInterior=1, EditRadiusi=3.0, EditRho=0.3)
    cases["disk_cs_iso_g32"] = dict(dcs, Ordis=7)
    cases["disk_cs_zdir_x_g32"] = dict(dcs, phi=0.0, theta=90.0)
    cases["disk_cs_zdir_z_fcc_g24"] = dict(dl, ComboBoxInterior=1, EditRadiusi=3.0, EditRho=0.3, Ordis=6, theta=0.0,
                                           phi=0.0)
    cases["cyl_cs_zdir_z_g32"] = dict(C.scaled(C.CYL_GAUSS, 32), Ordis=6, theta=0.0, phi=0.0, ComboBoxInterior=1,
                                      EditRadiusi=7.0, EditRho=0.3)
    cases["disk_cs_gauss_x_g24"] = dict(dg24, phi=0.0, theta=90.0, ComboBoxInterior=1, EditRadiusi=3.0, EditRho=0.3)
    cases["disk_cs_gauss_z_fcc_g16"] = dict(C.scaled(C.SPHERE_FCC, 16), ComboBoxParticle=2, EditRadius=2.0,
                                            Length=12.0, SigmaL=0.2, Ordis=0, theta=0.0, phi=0.0, EditDbeta=15.0,
                                            ComboBoxInterior=1, EditRadiusi=3.0, EditRho=0.3)
    # core/shell cylinders with the Gaussian orientation
    ccs = dict(ComboBoxInterior=1, EditRadiusi=7.0, EditRho=0.3)
    cases["cyl_cs_gauss_g24"] = dict(C.scaled(C.CYL_GAUSS, 24), **ccs)
    cases["cyl_cs_gauss_x_g16"] = dict(C.scaled(C.CYL_GAUSS_X, 16), **ccs)
    cases["cyl_cs_gauss_y_g16"] = dict(C.scaled(C.CYL_GAUSS, 16), phi=90.0, **ccs)
    cases["cyl_cs_gauss_z_g24"] = dict(C.scaled(C.CYL_GAUSS, 24), theta=0.0, phi=0.0, **ccs)
    ves = dict(C.scaled(C.SPHERE, 32), ComboBoxParticle=3, Length=14.0, SigmaL=0.15)
    cases["vesicle_iso_g32"] = dict(ves, iso=0.2)
    cases["vesicle_zdir_g32"] = dict(ves, Ordis=6)
    cases["vesicle_fcc_g24"] = dict(sph, ComboBoxParticle=3, Ordis=7, Length=12.0, SigmaL=0.15)
    # isotropic cylinders (exact average for short ones, factorised for long
    # ones), homogeneous and core/shell, alone and on a lattice
    cyl_iso = dict(C.scaled(C.CYL_GAUSS, 32), Ordis=7)
    cases["cyl_iso_g32"] = dict(cyl_iso)
    cases["cyl_iso_short_g24"] = dict(C.scaled(C.CYL_GAUSS, 24), Ordis=7, EditRadius=10.0, Length=15.0)
    cases["cyl_iso_cs_g32"] = dict(cyl_iso, ComboBoxInterior=1, EditRadiusi=7.0, EditRho=0.3)
    cases["cyl_iso_fcc_g24"] = dict(sph, ComboBoxParticle=1, Ordis=7, EditRadius=5.0, Length=30.0, SigmaL=0.1)
    cases["cyl_iso_cs_fcc_g24"] = dict(sph, ComboBoxParticle=1, Ordis=7, EditRadius=5.0, Length=30.0, SigmaL=0.1,
                                       ComboBoxInterior=1, EditRadiusi=7.0, EditRho=0.3)
    ell = dict(C.scaled(C.SPHERE, 32), ComboBoxParticle=5, Ordis=7)
    cases["ellipsoid_prolate_g32"] = dict(ell, Length=16.0)
    cases["ellipsoid_oblate_g32"] = dict(ell, Length=6.0, iso=0.1)
    cases["ellipsoid_fcc_g24"] = dict(sph, ComboBoxParticle=5, Ordis=7, Length=11.0)
    return cases


IGN_NEW_SWITCH = {"sphere_fcc_ignswitch_g24", "cyl_gauss_x_ignswitch_g16"}


def ign_cbs_for(p):
    # cylinder on BCT is rejected by the console's combination check; the
    # benchmark runs it with bIgnoreCbs (doCalculation(..., bIgnoreCbs=true))
    return 1 if (p.get("ComboBoxParticle") == 1 and p.get("LType") == 8) else 0


def rejected_cases():
    base = C.scaled(C.SPHERE, 8)
    return {
        "uca_small": dict(base, uca=0.005),
        "ucc_small": dict(base, ucc=0.0),
        "particle_default": {k: v for k, v in base.items() if k != "ComboBoxParticle"},
        "cyl_on_bct_checked": dict(C.scaled(C.bct_set(0), 8)),
        "ltype_invalid": dict(base, LType=25),
        "peak_invalid": dict(C.scaled(C.SPHERE_FCC, 8), ComboBoxPeak=9),
    }


def main():
    if not refbind.available():
        sys.exit("oracle/_ref/libscref.so not built (oracle/build_ref.sh)")
    # --only a,b: (re)generate just these image cases and merge them into
    # cases.json; the fit and rejection fixtures are left as they are
    only = None
    if "--only" in sys.argv:
        only = set(sys.argv[sys.argv.index("--only") + 1].split(","))
    out = {}
    for name, p in image_cases().items():
        if only is not None and name not in only:
            continue
        r = refbind.RefCalc(p)
        ign = ign_cbs_for(p)
        ins = 1 if name in IGN_NEW_SWITCH else 0
        rc, err = r.run(nthreads=8, ign_new_switch=ins, ign_cbs=ign)
        if rc != 0 and "INVALID CBParticle" in err and not ign:
            # the console's combination check rejects it: run as the benchmark
            # runs such combinations, with bIgnoreCbs
            r.close()
            ign = 1
            r = refbind.RefCalc(p)
            rc, err = r.run(nthreads=8, ign_new_switch=ins, ign_cbs=ign)
        assert rc == 0, (name, err)
        img = r.image()
        # per-pixel conditioning of the reference computation: spread of the
        # (reference-pinned) oracle under one-ulp math-library perturbations;
        # for the generic combinations the oracle does not restate,
        # the spread of the reference's own probe build (oracle/ref_probe.c)
        P0 = cpu_oracle.prepare(p, ign)
        if ins == 0 and cpu_oracle.supported(P0):
            cond = cpu_oracle.condition(p, ign_cbs=ign, nthreads=8)
        else:
            cond = refbind.condition(p, ign_new_switch=ins, ign_cbs=ign, nthreads=8)
        rec = {"image": img, "dims": np.array(r.dims()), "cond": cond.astype(np.float32)}
        for a in ARRAYS:
            rec[a] = r.array(a)
        for s in SCALARS:
            rec["s_" + s] = np.array(r.scalar(s))
        if p.get("LType", 12) != 12:
            pm2 = int(r.scalar("peakmax2"))
            rec["latpar1"] = r.latpar(1)[: pm2 + 1]
            rec["latpar2"] = r.latpar(2)[: pm2 + 1]
            rec["latpar3"] = r.latpar(3)[: pm2 + 1]
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **rec)
        out[name] = {"params": p, "ign_cbs": ign, "ign_new_switch": ins, "shape": list(img.shape),
                     "nonfinite": int((~np.isfinite(img)).sum()), "zeros": int((img == 0).sum()),
                     "ill_conditioned": int((cond > 1e-12).sum())}
        print(name, img.shape, "nonfinite", out[name]["nonfinite"], "zeros", out[name]["zeros"],
              "ill-conditioned", out[name]["ill_conditioned"])
        r.close()
    if only is not None:
        with open(os.path.join(HERE, "cases.json")) as f:
            allc = json.load(f)
        allc["images"].update(out)
        with open(os.path.join(HERE, "cases.json"), "w") as f:
            json.dump(allc, f, indent=1, sort_keys=True)
        return

    # fit cases: target = reference image * deterministic multiplicative noise
    fits = {}
    rng = np.random.default_rng(20261203)
    p = C.scaled(C.SPHERE, 32)
    r = refbind.RefCalc(p)
    r.run(nthreads=8)
    img = r.image()
    target = img * (1.0 + 0.05 * rng.standard_normal(img.shape))
    target[0, 0] = 0.0
    target[3, 5] = -1.0
    variants = {
        "plain": dict(bstop=0, border=0, nofit=()),
        "border_bstop": dict(bstop=4, border=3, nofit=()),
        "nofit_rects": dict(bstop=0, border=0, nofit=((2, 2, 10, 12), (30, 40, 50, 60))),
        "corner_threshold": dict(bstop=-1, border=0, nofit=()),
    }
    fit_params = dict(p, EditRadius=10.4)
    for vname, v in variants.items():
        rf = refbind.RefCalc(fit_params)
        chi2, cnt, nan, fqs = rf.fit(target, nthreads=8, bstop=v["bstop"], border=v["border"], nofit=v["nofit"])
        fits[vname] = {"chi2": chi2, "cnt": cnt, "nancnt": nan, "bstop": v["bstop"], "border": v["border"],
                       "nofit": [list(x) for x in v["nofit"]]}
        np.save(os.path.join(HERE, f"fit_{vname}_fqs.npy"), fqs)
        print("fit", vname, chi2, cnt, nan)
        rf.close()
    np.save(os.path.join(HERE, "fit_target.npy"), target)

    rej = {}
    for name, p in rejected_cases().items():
        r = refbind.RefCalc(p)
        rc, err = r.run(nthreads=1)
        rej[name] = {"params": p, "rc": rc, "error": err, "dims": r.dims()}
        print("rejected", name, repr(err))
        r.close()

    with open(os.path.join(HERE, "cases.json"), "w") as f:
        json.dump({"images": out, "fit": {"params": fit_params, "variants": fits}, "rejected": rej}, f, indent=1,
                  sort_keys=True)


if __name__ == "__main__":
    main()
