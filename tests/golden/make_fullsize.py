"""Generate the benchmark-size oracle fixtures tests/golden/fullsize_c{2,3,5}.npz.

The inputs are rebuilt from seeds by tests/fullsize_cases.py (here and on the
GPU machine); each fixture stores the rescaling (a, b) it was computed with
and oracle references only:

* c2 (3D Anderson L=128, NC=4096, NR=64): all NC moments of eight probe
  columns from the C restatement of the reference CPU path (oracle/kpm_cpu.c,
  itself checked against the NumPy oracle by the CPU tests);
* c3 (Haldane 256x256, NC=512, NR=16): the full moment matrix from the NumPy
  oracle's blocked kpm_2d (K_left=64, K_right=16, src/moment.jl:987-1088) and
  sigma_xy at 201 Fermi energies from its kubo_bastin_cond
  (src/applications/conductivity.jl:101-157);
* c5 (graphene 128x128, NC=1024, NR=16): the DOS-window loss, its target DOS,
  and its derivative along an onsite and a hopping direction, both exactly
  (the oracle's dual-number recurrence) and by central differences of oracle
  moments;
* x1 (Haldane 64x64, NC=256, NR=8): sigma_xy(Ef=0) and its exact derivative
  along random onsite energies, t1 and t2 (the oracle's dual-number kpm_2d,
  with the currents' own dependence on the hoppings).

Run from the repository root:  python tests/golden/make_fullsize.py [c2] [c3] [c5] [x1]
(the c3 reference takes several minutes on 8 cores).
"""
from __future__ import annotations

import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
for p in (ROOT, ROOT / "kpm.jl_gb300", ROOT / "tests"):
    sys.path.insert(0, str(p))

import fullsize_cases as fc  # noqa: E402
from oracle import cpu_port, kpm_oracle as ko  # noqa: E402

OUT = Path(__file__).resolve().parent


def make_c2():
    H = fc.c2_hamiltonian()
    a, b, _ = ko.normalizeH(H, center=True)
    Hn = fc.rescaled(H, a, b)
    psi = fc.c2_probes(Hn.shape[0])
    cols = fc.C2["cols"]
    t = time.time()
    mu = cpu_port.kpm1d_cpu(Hn, fc.C2["NC"], np.ascontiguousarray(psi[:, cols]))
    print(f"c2: C port {time.time() - t:.0f} s, a={a!r} b={b!r}")
    np.savez_compressed(OUT / "fullsize_c2.npz", a=a, b=b, cols=cols, mu=mu)


def make_c3():
    H, Jx, Jy, area = fc.c3_model()
    a, b, _ = ko.normalizeH(H, center=True)
    Hn = fc.rescaled(H, a, b)
    NH = Hn.shape[0]
    psi = fc.c3_probes(NH)
    t = time.time()
    mu = ko.kpm_2d(Hn, Jx, Jy, fc.C3["NC"], psi, psi, fc.C3["K_left"], fc.C3["K_right"])
    print(f"c3: oracle kpm_2d {time.time() - t:.0f} s, a={a!r} b={b!r}")
    sigma = np.array([ko.kubo_bastin_cond(mu, a, ef, b=b, NH=NH, area=area) for ef in fc.C3["Ef"]])
    np.savez_compressed(OUT / "fullsize_c3.npz", a=a, b=b, area=area, mu=mu, sigma=sigma)


def make_c5():
    H, Ht, psi = fc.c5_inputs()
    NC, a = fc.C5["NC"], fc.C5["a"]
    Phi, q = fc.dos_weights(NC, a, fc.C5["E"])

    def mean_moments(Hx):
        return ko.kpm_1d_doubling(Hx, NC, psi).real.mean(axis=0)

    def loss(Hx):
        r = Phi @ mean_moments(Hx)
        return float(q @ (r - rho_t) ** 2), r

    rho_t = Phi @ mean_moments(Ht)
    L0, rho = loss(H)
    g = Phi.T @ (2 * q * (rho - rho_t))
    exact, fd = [], []
    eps = 1e-5
    for D in fc.c5_directions(H):
        exact.append(float(ko.kpm_1d_tangent(H, D, NC, psi).real.mean(axis=0) @ g))
        fd.append((loss(H + eps * D)[0] - loss(H - eps * D)[0]) / (2 * eps))
    print(f"c5: L={L0:.6e} exact={exact} fd={fd}")
    np.savez_compressed(OUT / "fullsize_c5.npz", loss=L0, rho_t=rho_t, exact=np.array(exact),
                        fd=np.array(fd))


def make_x1():
    H, Jx, Jy, area, dirs = fc.x1_model()
    a, b, _ = ko.normalizeH(H, center=True)
    Hn = fc.rescaled_keep(H, a, b)
    NH, NC = Hn.shape[0], fc.X1["NC"]
    psi = fc.x1_probes(NH)
    mu = ko.kpm_2d(Hn, Jx, Jy, NC, psi, psi, NC, 16)
    sigma = ko.kubo_bastin_cond(mu, a, fc.X1["Ef"], b=b, NH=NH, area=area)
    dsig = []
    for dH, dJx, dJy in dirs:
        dmu = ko.kpm_2d_tangent(Hn, dH / a, Jx, dJx, Jy, dJy, NC, psi, psi)
        # sigma is linear in mu at fixed (a, b): its derivative is sigma(dmu)
        dsig.append(ko.kubo_bastin_cond(dmu, a, fc.X1["Ef"], b=b, NH=NH, area=area))
    print(f"x1: sigma={sigma!r} dsigma={dsig}")
    np.savez_compressed(OUT / "fullsize_x1.npz", a=a, b=b, area=area, sigma=sigma,
                        dsigma=np.array(dsig))


if __name__ == "__main__":
    which = sys.argv[1:] or ["c2", "c3", "c5", "x1"]
    for w in which:
        {"c2": make_c2, "c3": make_c3, "c5": make_c5, "x1": make_x1}[w]()
