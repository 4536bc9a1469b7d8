"""Seeded synthetic inputs for the benchmark configurations.

The production ensembles the reference infiles point at are not available, so
inputs with the same shapes and value distributions stand in for them:

* eigenvectors V_t: complex Gaussian (3 L^3 x nev) per timeslice, columns
  orthonormalised by a thin QR (``orthonormal=True``) or only normalised
  (``orthonormal=False``, used for the large benchmark volumes where a QR per
  timeslice would dominate set-up time; column norms and entry statistics are
  the same);
* perambulators: complex Gaussian, (4 nev Lt) x (Lt/dilT dilE 4) in the
  re-sorted matrix layout of src/Perambulator.cpp:53-64;
* noise: Z2 x Z2 entries (+-1 +- i)/sqrt(2), as RandomVector::set
  (src/RandomVector.cpp:7-27) produces them.

Infiles are written in the reference's syntax (infiles/*.in) and parsed by the
front end like any user infile.
"""
from __future__ import annotations

import os
import tempfile
from dataclasses import dataclass, field

import numpy as np

PION_RHO_OPERATORS = [  # infiles/pipi_I1.in: rho components, then the pion
    "g1.d0.p0,1,2,3,4", "g10.d0.p0,1,2,3,4", "g15.d0.p0,1,2,3,4",
    "g2.d0.p0,1,2,3,4", "g11.d0.p0,1,2,3,4", "g14.d0.p0,1,2,3,4",
    "g3.d0.p0,1,2,3,4", "g12.d0.p0,1,2,3,4", "g13.d0.p0,1,2,3,4",
    "g5.d0.p0,1,2,3,4",
]


@dataclass
class Workload:
    name: str
    Lt: int
    L: int
    nev: int
    n_rnd: int
    dilT: int  # time slices per dilution block (TB:<dilT>)
    dilE: int  # eigenvector interlace (EI:<dilE>)
    operators: list
    correlators: list
    seed: int = 1234
    orthonormal: bool = True
    description: str = ""
    extra: dict = field(default_factory=dict)  # further global settings, e.g. alpha1
    # Quark lines replacing the single default one (flavours with the same
    # dilution; n_rnd is then their total number of random vectors).
    quark_lines: tuple = ()

    @property
    def dim_row(self):
        return 3 * self.L ** 3

    def infile_text(self, start_config=1):
        lines = [f"Lt = {self.Lt}", f"Lx = {self.L}", f"Ly = {self.L}", f"Lz = {self.L}",
                 f"start_config = {start_config}", f"end_config = {start_config}",
                 f"number_of_eigen_vec = {self.nev}", "output_path = correlators"]
        lines += [f"{k} = {v}" for k, v in self.extra.items()]
        quarks = self.quark_lines or (
            f"u:{self.n_rnd}:TB:{self.dilT}:EI:{self.dilE}:DF:4:synthetic",)
        lines += ["[quarks]"] + [f"quark = {q}" for q in quarks] + ["[operator_lists]"]
        lines += [f"operator_list = {o}" for o in self.operators]
        lines += ["[correlator_lists]"]
        lines += [f"correlator_list = {c}" for c in self.correlators]
        return "\n".join(lines) + "\n"

    def write_infile(self, directory=None):
        d = directory or tempfile.mkdtemp(prefix=f"slaph_{self.name}_")
        path = os.path.join(d, f"{self.name}.in")
        with open(path, "w") as f:
            f.write(self.infile_text())
        return path

    def _rng(self, *key):
        return np.random.default_rng([self.seed, *key])

    def eigenvectors(self, t):
        """Timeslice t as (nev, 3L^3) C-order, i.e. column-major V_t."""
        rng = self._rng(1, t)
        K = self.dim_row
        a = rng.standard_normal((self.nev, 2 * K)).view(np.complex128)  # (nev, K)
        if self.orthonormal:
            q, _ = np.linalg.qr(a.T)
            return np.ascontiguousarray(q.T)
        a /= np.linalg.norm(a, axis=1, keepdims=True)
        return a

    def perambulator(self, r):
        """[cols][rows] (column-major storage of the re-sorted matrix)."""
        rng = self._rng(2, r)
        rows = 4 * self.nev * self.Lt
        cols = (self.Lt // self.dilT) * self.dilE * 4
        return rng.standard_normal((cols, 2 * rows)).view(np.complex128)

    def noise(self, r):
        rng = self._rng(3, r)
        n = self.Lt * 4 * self.nev
        s = 0.5 * np.sqrt(2.0)
        re = np.where(rng.random(n) < 0.5, -s, s)
        im = np.where(rng.random(n) < 0.5, -s, s)
        return re + 1j * im

    def flops_vdaggerv(self, n_computed_ops):
        return 8.0 * self.nev ** 2 * self.dim_row * n_computed_ops * self.Lt


# BASELINE configurations, restated.
CONFIGS = {
    # 4^3 x 8, Nev 16, T2 E4I F, |p|^2 <= 1, gamma_5 and gamma_0 gamma_5.  Four
    # random vectors: C4cD needs four mutually distinct indices, with two the
    # reference's inner_product throws (src/DilutedTrace.cpp:37-41).
    "cfg1_4x8": Workload(
        "cfg1_4x8", Lt=8, L=4, nev=16, n_rnd=4, dilT=2, dilE=4,
        operators=["g5.d0.p0,1", "g6.d0.p0,1"],
        correlators=["C2c:Q0:Op0:Q0:Op0:P0,1", "C2c:Q0:Op1:Q0:Op1:P0,1",
                     "C4cD:Q0:Op0:Q0:Op0:Q0:Op0:Q0:Op0:P0,1"],
        seed=101, description="4^3x8 Nev=16, C2c + C4cD"),
    # The same with the two random vectors BASELINE names: C4cD has no
    # admissible index combination (error path).
    "cfg1_4x8_2rnd": Workload(
        "cfg1_4x8_2rnd", Lt=8, L=4, nev=16, n_rnd=2, dilT=2, dilE=4,
        operators=["g5.d0.p0,1", "g6.d0.p0,1"],
        correlators=["C2c:Q0:Op0:Q0:Op0:P0,1", "C4cD:Q0:Op0:Q0:Op0:Q0:Op0:Q0:Op0:P0,1"],
        seed=101, description="4^3x8 Nev=16, 2 random vectors"),
    # VdaggerV only: 24^3 x 48, Nev 120, 27 momenta |p|^2 <= 3, four gammas.
    "cfg2_24x48_vdv": Workload(
        "cfg2_24x48_vdv", Lt=48, L=24, nev=120, n_rnd=2, dilT=16, dilE=8,
        operators=["g5.d0.p0,1,2,3", "g6.d0.p0,1,2,3", "g1.d0.p0,1,2,3", "g2.d0.p0,1,2,3"],
        correlators=["C2c:Q0:Op0:Q0:Op0:P0,1,2,3"],
        seed=202, orthonormal=True, description="24^3x48 Nev=120 VdaggerV, 27 momenta"),
    # Full pipi I=1 set at 32^3 x 64, Nev 220, 5 random vectors, T16 E8I F,
    # total momenta |P|^2 <= 4 (operators of infiles/pipi_I1.in).
    "cfg3_32x64_pipi": Workload(
        "cfg3_32x64_pipi", Lt=64, L=32, nev=220, n_rnd=5, dilT=16, dilE=8,
        operators=PION_RHO_OPERATORS,
        correlators=(["C2c:Q0:Op9:Q0:Op9:P0,1,2,3,4"]
                     + [f"C3c:Q0:Op9:Q0:Op{k}:Q0:Op9:P0,1,2,3,4" for k in range(9)]
                     + ["C4cD:Q0:Op9:Q0:Op9:Q0:Op9:Q0:Op9:P0,1,2,3,4",
                        "C4cB:Q0:Op9:Q0:Op9:Q0:Op9:Q0:Op9:P0,1,2,3,4",
                        "C4cV:Q0:Op9:Q0:Op9:Q0:Op9:Q0:Op9:P0,1,2,3,4"]),
        seed=303, orthonormal=False,
        description="32^3x64 Nev=220 pipi I=1: C2c C3c C4cB C4cD C4cV"),
}


def small_pipi(L=4, Lt=8, nev=16, n_rnd=5, dilT=4, dilE=4, seed=404):
    """The cfg3 diagram set on a small lattice (parity tests)."""
    return Workload(
        "pipi_small", Lt=Lt, L=L, nev=nev, n_rnd=n_rnd, dilT=dilT, dilE=dilE,
        operators=["g1.d0.p0,1", "g2.d0.p0,1", "g5.d0.p0,1"],
        correlators=["C2c:Q0:Op2:Q0:Op2:P0,1", "C3c:Q0:Op2:Q0:Op0:Q0:Op2:P0,1",
                     "C3c:Q0:Op2:Q0:Op1:Q0:Op2:P0,1",
                     "C4cD:Q0:Op2:Q0:Op2:Q0:Op2:Q0:Op2:P0,1",
                     "C4cB:Q0:Op2:Q0:Op2:Q0:Op2:Q0:Op2:P0,1",
                     "C4cV:Q0:Op2:Q0:Op2:Q0:Op2:Q0:Op2:P0,1"],
        seed=seed, description="pipi diagram set on a small lattice")


# Small case of the 32^3x64 diagram set for kernel profiles: 16^3 x 32, Nev 64,
# momenta |p|^2 <= 1.  Eigenvectors (400 MB) exceed L2; a few GB on the device.
CONFIGS["prof_16x32_pipi"] = Workload(
    "prof_16x32_pipi", Lt=32, L=16, nev=64, n_rnd=5, dilT=16, dilE=8,
    operators=[o.replace("p0,1,2,3,4", "p0,1") for o in PION_RHO_OPERATORS],
    correlators=(["C2c:Q0:Op9:Q0:Op9:P0,1"]
                 + [f"C3c:Q0:Op9:Q0:Op{k}:Q0:Op9:P0,1" for k in range(9)]
                 + ["C4cD:Q0:Op9:Q0:Op9:Q0:Op9:Q0:Op9:P0,1",
                    "C4cB:Q0:Op9:Q0:Op9:Q0:Op9:Q0:Op9:P0,1",
                    "C4cV:Q0:Op9:Q0:Op9:Q0:Op9:Q0:Op9:P0,1"]),
    seed=505, orthonormal=False, description="profiling case: 16^3x32 Nev=64 pipi")


def grouped_pipi(name, nev, dilE, seed):
    """The 32^3x64 operator and diagram set with momenta |p|^2 <= 1 on a 4^3x8
    lattice.  Its trace lists contain dense groups (every A operand group with
    every B group: 28 x 28 and 28 x 36) next to residual lists, so both trace
    paths of the mixed precision mode run."""
    return Workload(
        name, Lt=8, L=4, nev=nev, n_rnd=5, dilT=4, dilE=dilE,
        operators=[o.replace("p0,1,2,3,4", "p0,1") for o in PION_RHO_OPERATORS],
        correlators=(["C2c:Q0:Op9:Q0:Op9:P0,1"]
                     + [f"C3c:Q0:Op9:Q0:Op{k}:Q0:Op9:P0,1" for k in range(9)]
                     + ["C4cD:Q0:Op9:Q0:Op9:Q0:Op9:Q0:Op9:P0,1",
                        "C4cB:Q0:Op9:Q0:Op9:Q0:Op9:Q0:Op9:P0,1",
                        "C4cV:Q0:Op9:Q0:Op9:Q0:Op9:Q0:Op9:P0,1"]),
        seed=seed, description=f"pipi set, |p|^2 <= 1, 4^3x8, Nev {nev}, EI{dilE}")


CONFIGS["pipi_groups_e4"] = grouped_pipi("pipi_groups_e4", nev=16, dilE=4, seed=606)
CONFIGS["pipi_groups_e8"] = grouped_pipi("pipi_groups_e8", nev=32, dilE=8, seed=707)
