"""Generate the golden fixtures in this folder from the UNMODIFIED reference program.

The reference (CAPOW) ships no tests, data or expected outputs, so its own behaviour is captured
here: oracle/_ref/capow_ref is the reference sources compiled against single-rank MPI / FFTW / GSL
stand-ins (oracle/Makefile.ref). For each case this script writes a seeded catalogue and a
run_parameters.dat, runs the reference, and stores

  * the raw bin sums Pk0..Pk4, Nmodes (and 2-D bins) left in its globals by compute_periodic_power,
  * the scalars that passed through MPI_Allreduce (NPERIODIC, sum w, sum w v^n),
  * its output file and stdout text,
  * for the small cases, the painted grids (after the halo fold, before mean subtraction),

plus parameter-file and catalogue error cases (stdout text). Run from the repo root, where the
reference sources are mounted:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle as orc  # noqa: E402

CASES = [
    # name, params, n particles, seed, keep grids
    ("nn_los0", dict(NX=8, NY=8, NZ=8, InterpOrder=1, LOS=0, DoInterlacing=1, Momentum=0, NK=6, Maxk=0.05,
                     Odd_Multipoles=1), 200, 1, True),
    ("cic_los0_mom1", dict(NX=8, NY=10, NZ=6, InterpOrder=2, LOS=0, DoInterlacing=1, Momentum=1, NK=6, Maxk=0.05,
                           Odd_Multipoles=1), 300, 2, True),
    ("tsc_los3_mom1", dict(NX=12, NY=8, NZ=10, InterpOrder=3, LOS=3, DoInterlacing=1, Momentum=1, NK=8, Maxk=0.06,
                           Odd_Multipoles=1), 400, 3, True),
    ("tsc_los0_mom2", dict(NX=10, NY=10, NZ=10, InterpOrder=3, LOS=0, DoInterlacing=1, Momentum=2, NK=8,
                           Maxk=0.05, Odd_Multipoles=0), 400, 4, True),
    ("tsc_los1_2d", dict(NX=16, NY=16, NZ=16, InterpOrder=3, LOS=1, DoInterlacing=1, Momentum=0, NK=10, Maxk=0.1,
                         Output2D=1, NMU=4, Odd_Multipoles=1), 1000, 5, False),
    ("cic_los2_log", dict(NX=16, NY=12, NZ=20, InterpOrder=2, LOS=2, DoInterlacing=0, Momentum=4, NK=7, Mink=-2.0,
                          Maxk=-0.8, OutputLog=1, Odd_Multipoles=1), 1000, 6, False),
    ("tsc_c0like", dict(NX=32, NY=32, NZ=32, InterpOrder=2, LOS=0, DoInterlacing=1, Momentum=0, NK=16, Maxk=0.1,
                        Odd_Multipoles=0), 20000, 7, False),
    ("m8_los3", dict(NX=16, NY=16, NZ=16, InterpOrder=3, LOS=3, DoInterlacing=1, Momentum=8, NK=8, Maxk=0.05,
                     Odd_Multipoles=1), 2000, 8, False),
]

BOX = dict(XMIN=-3.0, XMAX=997.0, YMIN=0.0, YMAX=1000.0, ZMIN=10.0, ZMAX=510.0)


def catalogue(p, n, seed):
    rng = np.random.default_rng(seed)
    lo = np.array([p.XMIN, p.YMIN, p.ZMIN])
    hi = np.array([p.XMAX, p.YMAX, p.ZMAX])
    N = np.array([p.NX, p.NY, p.NZ])
    d = (hi - lo) / N
    pos = rng.uniform(lo[:, None], hi[:, None], size=(3, n))
    m = max(1, n // 16)
    for a in range(3):  # nodes and half cells exercise every edge rule
        pos[a, a * m:(a + 1) * m] = lo[a] + d[a] * rng.integers(0, N[a], m)
        pos[a, (a + 3) * m:(a + 4) * m] = lo[a] + d[a] * (rng.integers(0, N[a], m) + 0.5)
    vel = rng.normal(0.0, 300.0, size=(3, n))
    return pos, vel


def main():
    orc.build()
    if not orc.ref_available():
        raise SystemExit("oracle/_ref/capow_ref is not built (reference sources not mounted)")
    manifest = {}
    with tempfile.TemporaryDirectory() as td:
        for name, kw, n, seed, grids in CASES:
            p = orc.Params(**BOX, **kw)
            pos, vel = catalogue(p, n, seed)
            r = orc.run_ref_binary(p, os.path.join(td, name), *pos, *vel, grids=grids)
            assert r["returncode"] == 0, r["stdout"]
            d = r["dump"]
            out = dict(x=pos[0], y=pos[1], z=pos[2], vx=vel[0], vy=vel[1], vz=vel[2],
                       allreduce=d["allreduce"], Nmodes=d["Nmodes"])
            for k in ("Pk0", "Pk1", "Pk2", "Pk3", "Pk4", "Pk_2D", "Nmodes_2D"):
                if k in d:
                    out[k] = d[k]
            for k, g in r.get("grids", {}).items():
                out["grid_" + k] = g
            np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
            with open(os.path.join(HERE, f"{name}.out"), "w") as f:
                f.write(r["output"])
            with open(os.path.join(HERE, f"{name}.stdout"), "w") as f:
                f.write(r["stdout"])
            manifest[name] = dict(params=dataclass_dict(p), n=n, seed=seed)
            with open(os.path.join(HERE, f"{name}.stdout"), "w") as f:
                f.write(r["stdout"].replace(os.path.join(td, name, "data.txt"), "{DATAFILE}").replace(
                    os.path.join(td, name, "out.txt"), "{OUTFILE}"))
        # parameter-file error cases: the reference's stdout for each
        errs = {}
        good = orc.Params(**BOX, NX=8, NY=8, NZ=8)
        base = os.path.join(td, "base.dat")
        good.write_file(base)
        with open(base) as f:
            lines = f.read().splitlines()
        variants = {
            "missing_tag": [l for l in lines if not l.startswith("NK ")],
            "duplicate_tag": lines + ["NX 8"],
            "unknown_tag": lines + ["InputFormat 1"],
            "bad_los": [("LOS 7" if l.startswith("LOS ") else l) for l in lines],
            "bad_order": [("InterpOrder 4" if l.startswith("InterpOrder ") else l) for l in lines],
            "bad_nk": [("NK 0" if l.startswith("NK ") else l) for l in lines],
            "bad_box": [("XMAX -5.0" if l.startswith("XMAX ") else l) for l in lines],
            "bad_k": [("Maxk -1.0" if l.startswith("Maxk ") else l) for l in lines],
            "nmu_2d": [("Output2D 1" if l.startswith("Output2D ") else ("NMU 0" if l.startswith("NMU ") else l))
                       for l in lines],
            "comments_and_short_lines": ["% comment line", "lonely"] + lines + ["   ", "% trailing"],
        }
        cat = os.path.join(td, "c.txt")
        orc.write_catalogue(cat, [1.0], [20.0], [30.0], [0.0], [0.0], [0.0])
        import subprocess

        for k, ls in variants.items():
            pf = os.path.join(td, f"{k}.dat")
            with open(pf, "w") as f:
                f.write("\n".join(ls) + "\n")
            r = subprocess.run([orc.REF_BIN, pf, cat, "none", os.path.join(td, "o.txt")], capture_output=True,
                               text=True)
            errs[k] = dict(lines=ls, stdout=r.stdout.replace(pf, "{PARAMFILE}").replace(cat, "{DATAFILE}"),
                           returncode=r.returncode)
        # catalogue error: a malformed line
        badcat = os.path.join(td, "bad.txt")
        with open(badcat, "w") as f:
            f.write("# header\n1 20 30 4 5 6\n1 20 three 4 5 6\n")
        r = subprocess.run([orc.REF_BIN, base, badcat, "none", os.path.join(td, "o.txt")], capture_output=True,
                           text=True)
        errs["catalogue_bad_line"] = dict(lines=lines, catalogue="# header\n1 20 30 4 5 6\n1 20 three 4 5 6\n",
                                          stdout=r.stdout.replace(badcat, "{DATAFILE}"), returncode=r.returncode)
        oobcat = os.path.join(td, "oob.txt")
        with open(oobcat, "w") as f:
            f.write("1 20 30 4 5 6\n2 21 31 0 0 0\n-7.5 22 33 1 1 1\n5000 20 20 0 0 0\n")
        r = subprocess.run([orc.REF_BIN, base, oobcat, "none", os.path.join(td, "o.txt")], capture_output=True,
                           text=True)
        errs["catalogue_out_of_box"] = dict(lines=lines, catalogue="1 20 30 4 5 6\n2 21 31 0 0 0\n-7.5 22 33 1 1 1\n"
                                            "5000 20 20 0 0 0\n", stdout=r.stdout.replace(oobcat, "{DATAFILE}"),
                                            returncode=r.returncode)
        r = subprocess.run([orc.REF_BIN, base], capture_output=True, text=True)
        errs["usage"] = dict(stdout=r.stdout, returncode=r.returncode)
        with open(os.path.join(HERE, "param_errors.json"), "w") as f:
            json.dump(errs, f, indent=1)
    with open(os.path.join(HERE, "manifest.json"), "w") as f:
        json.dump(manifest, f, indent=1)
    print("wrote", len(CASES), "cases")


# survey-mode cases (Periodic 0, Survey 1; Cartesian input unless a case sets Coord_Type; number density from its
# column unless NBAR_Column < 0; FKP weights): name, params, data objects, random objects, seed
SURVEY_CASES = [
    ("sv_tsc_il_odd", dict(NX=32, NY=32, NZ=32, XMIN=100.0, XMAX=1100.0, YMIN=-500.0, YMAX=500.0, ZMIN=-500.0,
                           ZMAX=500.0, InterpOrder=3, DoInterlacing=1, NK=12, Maxk=0.09, Odd_Multipoles=1,
                           REDMININ=0.0, REDMAXIN=5.0, FKP_Pk=5000.0), 2000, 20000, 11),
    ("sv_cic_cut", dict(NX=24, NY=20, NZ=16, XMIN=-800.0, XMAX=-200.0, YMIN=300.0, YMAX=800.0, ZMIN=-250.0,
                        ZMAX=250.0, InterpOrder=2, DoInterlacing=0, NK=10, Maxk=0.12, Odd_Multipoles=0,
                        REDMININ=0.15, REDMAXIN=0.28, FKP_Pk=10000.0, X_Origin=10.0, Y_Origin=-20.0, Z_Origin=5.0),
     1500, 15000, 12),
    ("sv_nn_il", dict(NX=16, NY=16, NZ=16, XMIN=0.0, XMAX=600.0, YMIN=0.0, YMAX=600.0, ZMIN=-100.0, ZMAX=500.0,
                      InterpOrder=1, DoInterlacing=1, NK=8, Maxk=0.08, Odd_Multipoles=1, REDMININ=0.0, REDMAXIN=5.0,
                      FKP_Pk=3000.0, X_Origin=300.0, Y_Origin=300.0, Z_Origin=-200.0), 1000, 10000, 13),
    # the number density from the randoms' redshifts (compute_nbar, NBAR_Column < 0), observer at the centre
    ("sv_cic_nbar", dict(NX=24, NY=24, NZ=24, XMIN=-600.0, XMAX=600.0, YMIN=-600.0, YMAX=600.0, ZMIN=-600.0,
                         ZMAX=600.0, InterpOrder=2, DoInterlacing=1, NK=10, Maxk=0.1, Odd_Multipoles=0,
                         REDMININ=0.0, REDMAXIN=0.3, FKP_Pk=4000.0, NBAR_Column=-1, SkyArea=41253.0), 1500, 12000,
     14),
    # velocity surveys: the peculiar velocities from log-distance ratios, P_vv (Momentum 1) and the
    # density-velocity cross spectra. The reference's survey Momentum 2 writes its momentum grid before
    # allocating it (create_grids allocates ddg_mom only for Momentum not in {0, 2, 5}, src/main.c:1198) and
    # crashes; Momentum 3 runs the same cross-spectrum code (its norm, src/main.c:164-165, 184-186, is zero)
    ("sv_vv_tsc_il", dict(NX=24, NY=24, NZ=24, XMIN=50.0, XMAX=650.0, YMIN=-300.0, YMAX=300.0, ZMIN=-300.0,
                          ZMAX=300.0, InterpOrder=3, DoInterlacing=1, NK=10, Maxk=0.12, Odd_Multipoles=1,
                          REDMININ=0.0, REDMAXIN=5.0, FKP_Pk=4000.0, FKP_Pk_mom=5.0e9, Momentum=1), 1500, 6000, 15),
    ("sv_dv_cic_il", dict(NX=24, NY=20, NZ=16, XMIN=-700.0, XMAX=-100.0, YMIN=100.0, YMAX=600.0, ZMIN=-200.0,
                          ZMAX=200.0, InterpOrder=2, DoInterlacing=1, NK=10, Maxk=0.12, Odd_Multipoles=1,
                          REDMININ=0.0, REDMAXIN=5.0, FKP_Pk=4000.0, FKP_Pk_mom=5.0e9, FKP_Pk_cross=1.0e5,
                          Momentum=3, X_Origin=30.0, Y_Origin=-10.0, Z_Origin=0.0), 1500, 9000, 16),
    ("sv_dv3_tsc", dict(NX=16, NY=16, NZ=16, XMIN=100.0, XMAX=500.0, YMIN=-200.0, YMAX=200.0, ZMIN=-200.0,
                        ZMAX=200.0, InterpOrder=3, DoInterlacing=0, NK=8, Maxk=0.12, Odd_Multipoles=0,
                        REDMININ=0.0, REDMAXIN=5.0, FKP_Pk=4000.0, FKP_Pk_mom=5.0e9, FKP_Pk_cross=1.0e5,
                        Momentum=3), 1000, 6000, 17),
    # RA, Dec (degrees) and redshift input (Coord_Type 1): the reader's redshift-to-distance table and angle
    # conversion (src/read_data.c:267-291), the observer at the origin of the converted coordinates
    ("sv_radec_tsc_il", dict(NX=24, NY=24, NZ=24, XMIN=300.0, XMAX=900.0, YMIN=-300.0, YMAX=300.0, ZMIN=-300.0,
                             ZMAX=300.0, InterpOrder=3, DoInterlacing=1, NK=10, Maxk=0.12, Odd_Multipoles=1,
                             REDMININ=0.0, REDMAXIN=5.0, FKP_Pk=5000.0, Coord_Type=1), 1500, 12000, 18),
]


def to_radec(p, cat):
    """Cartesian positions (observer at the origin) as RA and Dec in degrees and redshift, in place of the first
    three columns: the redshift of each distance from the oracle's redshift-distance table."""
    L = orc._survey_lib()
    r = np.linalg.norm(cat[:, :3], axis=1)
    ra = np.degrees(np.arctan2(cat[:, 1], cat[:, 0])) % 360.0
    dec = np.degrees(np.arcsin(cat[:, 2] / r))
    z = np.array([L.orc_survey_redshift(p.Omega_m, float(v)) for v in r])
    out = cat.copy()
    out[:, 0], out[:, 1], out[:, 2] = ra, dec, z
    return out


def survey_catalogue(p, n, ncol, rng):
    """Objects uniform inside the grid less the reference's interpolation margin (src/read_data.c:193-204),
    weights in [0.5, 1.5], a smooth number density in the 5th column, zeros in the others."""
    d = np.array([(p.XMAX - p.XMIN) / p.NX, (p.YMAX - p.YMIN) / p.NY, (p.ZMAX - p.ZMIN) / p.NZ])
    lo = np.array([p.XMIN, p.YMIN, p.ZMIN]) + (p.InterpOrder - 1) * d
    hi = np.array([p.XMAX, p.YMAX, p.ZMAX]) - (p.InterpOrder - 1) * d - (0.5 * d if p.DoInterlacing else 0.0)
    pos = rng.uniform(lo + 1e-3 * d, hi - 1e-3 * d, size=(n, 3))
    w = rng.uniform(0.5, 1.5, n)
    nb = 1e-4 * (1.0 + 0.5 * np.sin(np.linalg.norm(pos, axis=1) / 200.0))
    out = np.concatenate([pos, w[:, None], nb[:, None], np.zeros((n, ncol - 5))], axis=1)
    if p.Momentum:  # log-distance ratios and their errors (data: 7th and 8th numbers; randoms: the 7th error)
        if ncol == 12:
            out[:, 6] = rng.normal(0.0, 0.05, n)
            out[:, 7] = rng.uniform(0.05, 0.1, n)
        else:
            out[:, 6] = rng.uniform(0.05, 0.1, n)
    return out


def main_survey():
    import subprocess

    orc.build()
    if not orc.ref_available():
        raise SystemExit("oracle/_ref/capow_ref is not built (reference sources not mounted)")
    manifest = {}
    with tempfile.TemporaryDirectory() as td:
        for name, kw, nd, nr, seed in SURVEY_CASES:
            p = orc.Params(**{"Periodic": 0, "Coord_Type": 0, "NBAR_Column": 5, "FKP_Column": -1, **kw,
                              "NOBJ_Max": max(nd, nr) + 10})
            rng = np.random.default_rng(seed)
            data, rand = survey_catalogue(p, nd, 12, rng), survey_catalogue(p, nr, 8, rng)
            if p.Coord_Type == 1:
                data, rand = to_radec(p, data), to_radec(p, rand)
            pf, df, rf, of, dump = (os.path.join(td, f"{name}.{e}") for e in ("dat", "data", "rand", "out", "dump"))
            p.write_file(pf)
            np.savetxt(df, data, fmt="%.17g")
            np.savetxt(rf, rand, fmt="%.17g")
            r = subprocess.run([orc.REF_BIN, pf, df, rf, of], capture_output=True, text=True,
                               env=dict(os.environ, CAPOW_REF_DUMP=dump))
            assert r.returncode == 0, r.stdout
            dd = orc.parse_dump(dump)
            np.savez_compressed(os.path.join(HERE, f"{name}.npz"), data=data, rand=rand, Nmodes=dd["Nmodes"],
                                **{k: dd[k] for k in ("Pk0", "Pk1", "Pk2", "Pk3", "Pk4")})
            with open(os.path.join(HERE, f"{name}.out"), "w") as f:
                f.write(open(of).read())
            with open(os.path.join(HERE, f"{name}.stdout"), "w") as f:
                f.write(r.stdout.replace(df, "{DATAFILE}").replace(rf, "{RANDFILE}").replace(of, "{OUTFILE}"))
            manifest[name] = dict(params=dataclass_dict(p), ndata=nd, nrand=nr, seed=seed)
    with open(os.path.join(HERE, "survey_manifest.json"), "w") as f:
        json.dump(manifest, f, indent=1)
    print("wrote", len(SURVEY_CASES), "survey cases")


def dataclass_dict(p):
    import dataclasses

    return dataclasses.asdict(p)


if __name__ == "__main__":
    if "--survey" in sys.argv:
        main_survey()
    else:
        main()
