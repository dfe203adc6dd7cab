"""Output files in the reference's layout (Source/Dump_Data.F90) and their reader
(the cursor walk of Analyze/NEGF_ReadData.m).  CPU only."""
import os

import numpy as np

from nonequilibriumgreensfunction_gb300 import dump


def test_es11_4_matches_fortran_edit_descriptor():
    assert dump.es11_4(1.0) == " 1.0000E+00"
    assert dump.es11_4(-0.000123456) == "-1.2346E-04"
    assert dump.es11_4(0.0) == " 0.0000E+00"
    assert dump.es11_4(6.02214e23) == " 6.0221E+23"
    assert dump.es11_4(1.23456e-100) == " 1.2346-100"      # three-digit exponent: no 'E'
    assert dump.es11_4(-9.99996e5) == "-1.0000E+06"        # rounding carries into the exponent
    assert all(len(dump.es11_4(v)) == 11 for v in (1e-300, -1e300, 3.3, -0.5))


def _record(npx=3, npy=2, npz=2, n_e=5, poisson=True, spin=True, seed=0):
    rng = np.random.default_rng(seed)
    site = lambda: rng.normal(size=(npx, npy, npz))        # noqa: E731
    per_e = lambda: rng.normal(size=n_e)                   # noqa: E731
    rec = dict(npx=npx, npy=npy, npz=npz, norb=4, muT=0.0, eMin=-0.3, eMax=0.3, eStpnum=n_e, deltaE=0.15,
               mu=np.array([0.005, -0.005]), channelType=0, a0=1.0, abPhi=0.5, corrLength=0.0,
               disorderStrength=0.1, RhoN=site(), RhoP=site(), DeltaR=np.zeros((npx, npy, npz)),
               EDensity=per_e(), HDensity=per_e(), T12=per_e(), Modec1=per_e(), Modec2=per_e(),
               EAxis=np.linspace(-0.3, 0.3, n_e), ContactCurrent=rng.normal(size=2) * 1e-6,
               Jx=site() * 1e-5, Jy=site() * 1e-5, Jz=site() * 1e-5, DOSc1=per_e(), DOSc2=per_e())
    if poisson:
        rec["Phi"], rec["ro"] = site(), site()
    if spin:
        rec["SigX"], rec["SigY"], rec["SigZ"] = site(), site(), site()
    return rec


def test_reference_files_round_trip(tmp_path):
    rec = _record()
    paths = dump.write_reference_files(str(tmp_path), rec)
    names = sorted(os.path.basename(p) for p in paths)
    assert names == ["Greens.txt", "Poissons.txt", "SigExp.txt", "Transmissions.txt", "scalars.txt"]
    back = dump.read_reference_files(str(tmp_path))
    for k in ("npx", "npy", "npz", "norb", "eStpnum", "channelType"):
        assert back[k] == rec[k]
    es_fields = ("RhoN", "RhoP", "EDensity", "HDensity", "T12", "Modec1", "Modec2", "DOSc1", "DOSc2", "Phi", "ro",
                 "SigX", "SigY", "SigZ")
    for k in es_fields:                                   # ES11.4: 5 significant digits
        assert np.allclose(back[k], rec[k], rtol=5.1e-5, atol=0), k
    for k in ("EAxis", "ContactCurrent", "Jx", "Jy", "Jz"):   # list-directed: full precision
        assert np.array_equal(back[k], rec[k]), k
    assert np.array_equal(back["mu"], np.array([0.005, -0.005]))


def test_file_layout_follows_dump_data(tmp_path):
    rec = _record(npx=2, npy=2, npz=1, n_e=3, poisson=False, spin=False)
    dump.write_reference_files(str(tmp_path), rec)
    g = open(tmp_path / "Greens.txt").read().split("\n")
    ns = 4
    assert len([x for x in g if x]) == 3 * ns            # RhoN/RhoP interleaved, then DeltaR
    assert g[0] == dump.es11_4(rec["RhoN"][0, 0, 0]) and g[1] == dump.es11_4(rec["RhoP"][0, 0, 0])
    assert g[2] == dump.es11_4(rec["RhoN"][0, 1, 0])      # z fastest, then y, then x
    t = [x for x in open(tmp_path / "Transmissions.txt").read().split("\n") if x]
    assert len(t) == 2 * 3 + 3 + 2 * 3 + 3 + 2 + 3 * ns + 2 * 3
    s = [x for x in open(tmp_path / "scalars.txt").read().split("\n") if x]
    assert s[0] == "           2" and len(s) == 15      # channelType 0: no a0 line
    assert not os.path.exists(tmp_path / "Poissons.txt")


def test_npz_is_lossless(tmp_path):
    rec = _record()
    dump.write_npz(str(tmp_path / "run.npz"), rec)
    back = dump.read_npz(str(tmp_path / "run.npz"))
    for k, v in rec.items():
        assert np.array_equal(np.asarray(back[k]), np.asarray(v)), k


def test_resolved_files_follow_dump_data(tmp_path):
    """ERCD.txt: per site (z fastest), per energy the four values ERJx, ERJy, ERJz, ERRhon;
    ORCD.txt: per site the norb^2 pair triples (ORJx, ORJy, ORJz), then the norb ORRhon
    values (Source/Dump_Data.F90:100-132)."""
    npx, npy, npz, n_e = 2, 2, 1, 3
    rng = np.random.default_rng(3)
    rec = _record(npx=npx, npy=npy, npz=npz, n_e=n_e, poisson=False, spin=False)
    for k in ("ERJx", "ERJy", "ERJz", "ERRhon"):
        rec[k] = rng.normal(size=(npx, npy, npz, n_e))
    for k in ("ORJx", "ORJy", "ORJz"):
        rec[k] = rng.normal(size=(npx, npy, npz, 16))
    rec["ORRhon"] = rng.normal(size=(npx, npy, npz, 4))
    names = sorted(os.path.basename(p) for p in dump.write_reference_files(str(tmp_path), rec))
    assert "ERCD.txt" in names and "ORCD.txt" in names
    e = [x for x in open(tmp_path / "ERCD.txt").read().split("\n") if x]
    assert len(e) == 4 * n_e * npx * npy * npz
    assert e[0] == dump.es11_4(rec["ERJx"][0, 0, 0, 0]) and e[3] == dump.es11_4(rec["ERRhon"][0, 0, 0, 0])
    assert e[4] == dump.es11_4(rec["ERJx"][0, 0, 0, 1])                 # next energy
    assert e[4 * n_e] == dump.es11_4(rec["ERJx"][0, 1, 0, 0])           # next site: y
    o = [x for x in open(tmp_path / "ORCD.txt").read().split("\n") if x]
    per_site = 3 * 16 + 4
    assert len(o) == per_site * npx * npy * npz
    assert o[1] == dump.es11_4(rec["ORJy"][0, 0, 0, 0]) and o[3] == dump.es11_4(rec["ORJx"][0, 0, 0, 1])
    assert o[48] == dump.es11_4(rec["ORRhon"][0, 0, 0, 0])
    back = dump.read_reference_files(str(tmp_path))
    for k in ("ERJx", "ERJy", "ERJz", "ERRhon", "ORJx", "ORJy", "ORJz", "ORRhon"):
        assert back[k].shape == rec[k].shape
        assert np.allclose(back[k], rec[k], rtol=5.1e-5, atol=0), k
