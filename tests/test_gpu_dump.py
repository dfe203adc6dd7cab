"""A device run written in the reference's output layout and read back the MATLAB
reader's way matches the oracle to the files' precision (ES11.4: 5 digits)."""
import numpy as np
import pytest

from oracle import negf_oracle as O
from nonequilibriumgreensfunction_gb300 import Solver, dump, scf
from nonequilibriumgreensfunction_gb300 import hamiltonian as HB

pytestmark = pytest.mark.gpu


def test_device_run_to_reference_files(need_gpu, tmp_path):
    npx, npy, npz = 5, 3, 2
    htotd, hopx = HB.ti_wire(npx, npy, npz, W=0.1, seed=2, flux=0.5, zeeman=0.01)
    mu = (0.005, -0.005)
    energies = np.linspace(-0.3, 0.3, 7)
    de = energies[1] - energies[0]
    f1 = np.array([scf.occupation(e, mu[0], 0.025) for e in energies])
    f2 = np.array([scf.occupation(e, mu[1], 0.025) for e in energies])
    shape = (npx, npy, npz, 1)
    rn, rp = np.zeros(shape, order="F"), np.zeros(shape, order="F")
    spin = [np.zeros(shape, order="F") for _ in range(3)]
    cur = [np.zeros(shape, order="F") for _ in range(3)]
    with Solver(npx, npy, npz, max_batch=4, eta=1e-5, sr_tol=1e-10, calc_spin=True, calc_currents=True) as s:
        s.set_hamiltonian(htotd, hopx)
        out = s.solve_batch(energies, f1, f2, de, rho_n=rn, rho_p=rp, spin=spin, currents=cur)
    rec = dump.record_from_sweep(npx, npy, npz, energies, de, mu, 0.0, out, rn[..., 0], rp[..., 0], f1=f1, f2=f2,
                                 spin=[a[..., 0] for a in spin], currents=[a[..., 0] for a in cur], flux=0.5,
                                 disorder=0.1)
    dump.write_reference_files(str(tmp_path), rec)
    back = dump.read_reference_files(str(tmp_path))
    opt = O.SolveOptions(eta=1e-5, sr_tol=1e-10, kT=0.025, calc_spin=True)
    want_t = []
    want_rn = np.zeros((npx, npy, npz))
    want_j = [np.zeros((npx, npy, npz)) for _ in range(3)]
    for e in energies:
        r = O.energy_sweep(htotd, hopx, float(e), mu, de, npy, npz, opt, calc_currents=True)
        want_t.append(r["T12"])
        want_rn += r["RhoN"]
        for i, k in enumerate(("Jx", "Jy", "Jz")):
            want_j[i] += r[k]
    assert np.allclose(back["T12"], want_t, rtol=6e-5, atol=1e-9)
    assert np.allclose(back["RhoN"], want_rn, rtol=6e-5, atol=0)
    for i, k in enumerate(("Jx", "Jy", "Jz")):           # list-directed: full precision
        assert np.abs(back[k] - want_j[i]).max() <= 1e-6 * np.abs(want_j[i]).max()
    assert np.array_equal(back["EAxis"], energies)
