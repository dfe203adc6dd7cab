"""Output files of a run in the reference's layout (Source/Dump_Data.F90:1-152), and a
reader that walks them the way the reference's MATLAB reader does
(Analyze/NEGF_ReadData.m:13-176).

The reference writes one value per line: numbers with ``FORMAT(ES11.4)`` (four decimals,
``Dump_Data.F90:152``) and the rest list-directed (``WRITE(13, *)``), whose layout the
Fortran standard leaves to the compiler.  ``write_reference_files`` reproduces the ES11.4
fields character for character (including the E-less form of three-digit exponents) and
writes list-directed integers right-justified in 12 columns and list-directed reals with
17 significant digits; the MATLAB reader parses both with ``load``.  ES11.4 keeps only five
significant digits, so a lossless ``.npz`` of the same record (``write_npz``) sits beside
it for parity work.

A record is a dict with the arrays of NEGF_Module (site arrays (npx, npy, npz), per-energy
arrays (n_e,)) and the scalars of scalars.txt; ``record_from_sweep`` builds one from a
batched solve.
"""
from __future__ import annotations

import os

import numpy as np

SCALAR_KEYS = ("npx", "npy", "npz", "norb", "muT", "eMin", "eMax", "eStpnum", "deltaE", "mu",
               "channelType", "a0", "abPhi", "corrLength", "disorderStrength")


def es11_4(v: float) -> str:
    """Fortran ``ES11.4``: d.dddd with a signed two-digit exponent, or three digits and no
    'E' when the exponent exceeds 99 in magnitude (Fortran 2008, 10.7.2.3.2)."""
    v = float(v)
    if not np.isfinite(v):
        return ("%11s" % ("NaN" if np.isnan(v) else ("-Infinity" if v < 0 else "Infinity")))
    s = "%.4E" % v                        # correctly rounded, as Fortran's formatted output
    mant, exp = s.split("E")
    e = int(exp)
    if abs(e) <= 99:
        body = "%sE%s%02d" % (mant, "-" if e < 0 else "+", abs(e))
    else:
        body = "%s%s%03d" % (mant, "-" if e < 0 else "+", abs(e))
    return "%11s" % body


def list_int(v: int) -> str:
    return "%12d" % int(v)


def list_real(v: float) -> str:
    return "%25.16E" % float(v)


def _site_loop(npx, npy, npz):
    for x in range(npx):
        for y in range(npy):
            for z in range(npz):
                yield x, y, z


def write_reference_files(outdir: str, rec: dict) -> list:
    """Write scalars.txt, Greens.txt, Transmissions.txt and, when present in the record,
    Poissons.txt (Phi, ro), ERCD.txt (ERJx/y/z, ERRhon: (npx, npy, npz, n_e)), ORCD.txt
    (ORJx/y/z: (npx, npy, npz, norb**2), ORRhon: (npx, npy, npz, norb)) and SigExp.txt
    (SigX/Y/Z), in Dump_Data's order.  Returns the paths written."""
    os.makedirs(outdir, exist_ok=True)
    npx, npy, npz = int(rec["npx"]), int(rec["npy"]), int(rec["npz"])
    out = []

    def put(name, lines):
        path = os.path.join(outdir, name)
        with open(path, "w") as f:
            f.write("\n".join(lines) + "\n")
        out.append(path)

    # scalars.txt (:6-25)
    s = [list_int(npx), list_int(npy), list_int(npz), list_int(rec["norb"]), es11_4(rec["muT"]),
         es11_4(rec["eMin"]), es11_4(rec["eMax"]), list_int(rec["eStpnum"]), es11_4(rec["deltaE"])]
    s += [es11_4(m) for m in rec["mu"]]
    s.append(list_int(rec["channelType"]))
    if int(rec["channelType"]) == 1:
        s.append(list_real(rec["a0"]))
    s += [list_real(rec["abPhi"]), es11_4(rec["corrLength"]), es11_4(rec["disorderStrength"])]
    put("scalars.txt", s)

    # Greens.txt (:27-46): RhoN, RhoP interleaved per site, then DeltaR
    g = []
    for x, y, z in _site_loop(npx, npy, npz):
        g.append(es11_4(rec["RhoN"][x, y, z]))
        g.append(es11_4(rec["RhoP"][x, y, z]))
    delta = rec.get("DeltaR")
    if delta is None:
        delta = np.zeros((npx, npy, npz))     # pairing potential: zero outside the BdG models
    for x, y, z in _site_loop(npx, npy, npz):
        g.append(es11_4(delta[x, y, z]))
    put("Greens.txt", g)

    # Transmissions.txt (:48-85)
    n_e = int(rec["eStpnum"])
    t = []
    for i in range(n_e):
        t += [es11_4(rec["EDensity"][i]), es11_4(rec["HDensity"][i])]
    t += [es11_4(rec["T12"][i]) for i in range(n_e)]
    for i in range(n_e):
        t += [es11_4(rec["Modec1"][i]), es11_4(rec["Modec2"][i])]
    t += [list_real(rec["EAxis"][i]) for i in range(n_e)]
    t += [list_real(c) for c in rec["ContactCurrent"]]
    jx, jy, jz = (rec.get(k) for k in ("Jx", "Jy", "Jz"))
    zero = np.zeros((npx, npy, npz))
    for x, y, z in _site_loop(npx, npy, npz):
        for j in (jx, jy, jz):
            t.append(list_real((zero if j is None else j)[x, y, z]))
    for i in range(n_e):
        t += [es11_4(rec["DOSc1"][i]), es11_4(rec["DOSc2"][i])]
    put("Transmissions.txt", t)

    if rec.get("Phi") is not None:           # Poissons.txt (:87-99)
        p = []
        for x, y, z in _site_loop(npx, npy, npz):
            p += [es11_4(rec["Phi"][x, y, z]), es11_4(rec["ro"][x, y, z])]
        put("Poissons.txt", p)
    if rec.get("ERJx") is not None:          # ERCD.txt (:100-114): per site, per energy
        er = [rec[k] for k in ("ERJx", "ERJy", "ERJz", "ERRhon")]
        lines = []
        for x, y, z in _site_loop(npx, npy, npz):
            for i in range(n_e):
                lines += [es11_4(a[x, y, z, i]) for a in er]
        put("ERCD.txt", lines)
    if rec.get("ORJx") is not None:          # ORCD.txt (:116-132): pairs, then orbitals
        norb = int(rec["norb"])
        oj = [rec[k] for k in ("ORJx", "ORJy", "ORJz")]
        lines = []
        for x, y, z in _site_loop(npx, npy, npz):
            for q in range(norb * norb):
                lines += [es11_4(a[x, y, z, q]) for a in oj]
            lines += [es11_4(rec["ORRhon"][x, y, z, o]) for o in range(norb)]
        put("ORCD.txt", lines)
    if rec.get("SigX") is not None:          # SigExp.txt (:134-146)
        sp = []
        for x, y, z in _site_loop(npx, npy, npz):
            sp += [es11_4(rec["SigX"][x, y, z]), es11_4(rec["SigY"][x, y, z]), es11_4(rec["SigZ"][x, y, z])]
        put("SigExp.txt", sp)
    return out


def _load(path):
    vals = []
    with open(path) as f:
        for line in f:
            line = line.strip()
            if not line:
                continue
            # three-digit exponents without 'E' (ES11.4 beyond 1e+-99): d.dddd+eee
            if "E" not in line.upper() and ("+" in line[1:] or "-" in line[1:]):
                k = max(line.rfind("+"), line.rfind("-"))
                line = line[:k] + "E" + line[k:]
            vals.append(float(line))
    return np.array(vals)


def read_reference_files(outdir: str) -> dict:
    """Parse the files the way Analyze/NEGF_ReadData.m:13-176 does (a cursor over the
    numbers of each file)."""
    r = _load(os.path.join(outdir, "scalars.txt"))
    c = 0
    rec = {}
    for k in ("npx", "npy", "npz", "norb"):
        rec[k] = int(r[c]); c += 1
    for k in ("muT", "eMin", "eMax"):
        rec[k] = r[c]; c += 1
    rec["eStpnum"] = int(r[c]); c += 1
    rec["deltaE"] = r[c]; c += 1
    rec["mu"] = r[c:c + 2].copy(); c += 2
    rec["channelType"] = int(r[c]); c += 1
    if rec["channelType"] == 1:
        rec["a0"] = r[c]; c += 1
    else:
        rec["a0"] = 1.0
    rec["abPhi"] = r[c]; c += 1
    rec["corrLength"] = r[c]; c += 1
    rec["disorderStrength"] = r[c]; c += 1
    npx, npy, npz, n_e = rec["npx"], rec["npy"], rec["npz"], rec["eStpnum"]
    ns = npx * npy * npz

    def sites(flat, per):
        # flat values in the x, y, z loop order (z fastest), `per` interleaved fields
        a = flat.reshape(npx, npy, npz, per)
        return [a[..., i] for i in range(per)]

    g = _load(os.path.join(outdir, "Greens.txt"))
    rec["RhoN"], rec["RhoP"] = sites(g[:2 * ns], 2)
    if g.size >= 3 * ns:
        rec["DeltaR"] = sites(g[2 * ns:3 * ns], 1)[0]
    t = _load(os.path.join(outdir, "Transmissions.txt"))
    c = 0
    ed = t[c:c + 2 * n_e].reshape(n_e, 2); c += 2 * n_e
    rec["EDensity"], rec["HDensity"] = ed[:, 0].copy(), ed[:, 1].copy()
    rec["T12"] = t[c:c + n_e].copy(); c += n_e
    mo = t[c:c + 2 * n_e].reshape(n_e, 2); c += 2 * n_e
    rec["Modec1"], rec["Modec2"] = mo[:, 0].copy(), mo[:, 1].copy()
    rec["EAxis"] = t[c:c + n_e].copy(); c += n_e
    rec["ContactCurrent"] = t[c:c + 2].copy(); c += 2
    rec["Jx"], rec["Jy"], rec["Jz"] = sites(t[c:c + 3 * ns], 3); c += 3 * ns
    do = t[c:c + 2 * n_e].reshape(n_e, 2); c += 2 * n_e
    rec["DOSc1"], rec["DOSc2"] = do[:, 0].copy(), do[:, 1].copy()
    pp = os.path.join(outdir, "Poissons.txt")
    if os.path.exists(pp):
        rec["Phi"], rec["ro"] = sites(_load(pp), 2)
    ep = os.path.join(outdir, "ERCD.txt")
    if os.path.exists(ep):
        a = _load(ep).reshape(npx, npy, npz, n_e, 4)
        for f, k in enumerate(("ERJx", "ERJy", "ERJz", "ERRhon")):
            rec[k] = a[..., f].copy()
    op = os.path.join(outdir, "ORCD.txt")
    if os.path.exists(op):
        no = rec["norb"]
        a = _load(op).reshape(npx, npy, npz, 3 * no * no + no)
        pairs = a[..., :3 * no * no].reshape(npx, npy, npz, no * no, 3)
        for f, k in enumerate(("ORJx", "ORJy", "ORJz")):
            rec[k] = pairs[..., f].copy()
        rec["ORRhon"] = a[..., 3 * no * no:].copy()
    sp = os.path.join(outdir, "SigExp.txt")
    if os.path.exists(sp):
        rec["SigX"], rec["SigY"], rec["SigZ"] = sites(_load(sp), 3)
    return rec


def write_npz(path: str, rec: dict) -> None:
    """Lossless copy of a record (every array in float64 / int64)."""
    np.savez(path, **{k: np.asarray(v) for k, v in rec.items() if v is not None})


def read_npz(path: str) -> dict:
    with np.load(path) as z:
        return {k: (z[k].item() if z[k].ndim == 0 else z[k]) for k in z.files}


def record_from_sweep(npx, npy, npz, energies, dE, mu, mu_t, out, rho_n, rho_p, f1=None, f2=None,
                      spin=None, currents=None, flux=0.0, disorder=0.0, norb=4, phi=None, ro=None,
                      er=None, orb=None):
    """Assemble a record from a batched solve of one Hamiltonian slot: ``out`` is the dict
    Solver.solve_batch returns for ``energies`` (in order), rho_n/rho_p/spin/currents the
    slot's (npx, npy, npz) sums, er = (ERJx, ERJy, ERJz, ERRhon) the (npx, npy, npz, n_e)
    energy-resolved arrays and orb = (ORJx, ORJy, ORJz, ORRhon) the slot's orbital-resolved
    ones.  With the per-energy occupations f1, f2, ContactCurrent is the sum over energies
    of Calculate_Observables.F90:102-103 (zero without them)."""
    energies = np.asarray(energies, dtype=np.float64)
    de = np.broadcast_to(np.asarray(dE, dtype=np.float64), energies.shape)
    contact_current = np.zeros(2)
    if f1 is not None and f2 is not None:
        q, h = 1.602e-19, 6.626e-34                       # Source/Constants.F90:4-6
        for i in range(energies.size):
            contact_current[0] += q * de[i] / h * (out["T12"][i] * (f2[i] - f1[i]))
            contact_current[1] += q * de[i] / h * (out["T12"][i] * (f1[i] - f2[i]))
    rec = dict(npx=npx, npy=npy, npz=npz, norb=norb, muT=mu_t, eMin=float(energies.min()),
               eMax=float(energies.max()), eStpnum=int(energies.size), deltaE=float(de[0]),
               mu=np.asarray(mu, dtype=np.float64), channelType=0, a0=1.0, abPhi=float(flux),
               corrLength=0.0, disorderStrength=float(disorder),
               RhoN=np.asarray(rho_n), RhoP=np.asarray(rho_p), DeltaR=np.zeros((npx, npy, npz)),
               EDensity=out["EDensity"], HDensity=out["HDensity"], T12=out["T12"], Modec1=out["Modec1"],
               Modec2=out["Modec2"], EAxis=energies, ContactCurrent=contact_current,
               DOSc1=out["DOSc1"], DOSc2=out["DOSc2"])
    if currents is not None:
        rec["Jx"], rec["Jy"], rec["Jz"] = currents
    if spin is not None:
        rec["SigX"], rec["SigY"], rec["SigZ"] = spin
    if phi is not None:
        rec["Phi"], rec["ro"] = phi, ro
    if er is not None:
        rec["ERJx"], rec["ERJy"], rec["ERJz"], rec["ERRhon"] = er
    if orb is not None:
        rec["ORJx"], rec["ORJy"], rec["ORJz"], rec["ORRhon"] = orb
    return rec
