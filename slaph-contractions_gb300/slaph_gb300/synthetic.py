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
    # > 0: timeslice t has the eigenvectors of timeslice t % v_period, so that
    # a workload whose eigenvectors exceed host memory needs only v_period of
    # them; every timeslice is still copied and computed.
    v_period: int = 0
    # > 0: the engine streams the eigenvectors through this many device slots
    # (slaph_engine_set_eigenvector_slots) instead of keeping all resident.
    eigenvector_slots: int = 0
    # True: factors built per block pair (slaph_engine_set_factor_lifetime),
    # for workloads whose factors of a whole configuration exceed the device.
    factors_per_block_pair: bool = False

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
        if self.v_period > 0:
            t %= self.v_period
        rng = self._rng(1, t)
        K = self.dim_row
        a = rng.standard_normal((self.nev, 2 * K)).view(np.complex128)  # (nev, K)
        if self.orthonormal:
            q, _ = np.linalg.qr(a.T)
            return np.ascontiguousarray(q.T)
        a /= np.linalg.norm(a, axis=1, keepdims=True)
        return a

    def gauge_links(self, t):
        """Random SU(3) links of timeslice t in the layout Engine.set_gauge
        takes: complex (L^3, 3, 9), site x L^2 + y L + z, directions x, y, z,
        each 3x3 matrix column-major.  Rows u1, u2 orthonormalised from complex
        Gaussians and u3 = conj(u1 x u2), which puts the matrix in SU(3)."""
        if self.v_period > 0:
            t %= self.v_period
        rng = self._rng(4, t)
        n = self.L ** 3 * 3
        z = rng.standard_normal((n, 2, 3)) + 1j * rng.standard_normal((n, 2, 3))
        u1 = z[:, 0] / np.linalg.norm(z[:, 0], axis=1, keepdims=True)
        u2 = z[:, 1] - np.sum(np.conj(u1) * z[:, 1], axis=1, keepdims=True) * u1
        u2 /= np.linalg.norm(u2, axis=1, keepdims=True)
        u3 = np.conj(np.cross(u1, u2))
        M = np.stack([u1, u2, u3], axis=1)  # M[a, b] = u_a[b]
        return np.ascontiguousarray(M.transpose(0, 2, 1)).reshape(self.L ** 3, 3, 9)

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
# 4 dilE = 64: one left matrix per product tile, four k-tiles per product
CONFIGS["pipi_groups_e16"] = grouped_pipi("pipi_groups_e16", nev=32, dilE=16, seed=808)


# 48^3 x 96, Nev 220 (eigenvectors 112 GB, streamed per timeslice): the pipi
# I=1 set of the 32^3 x 64 workload, the KK set of infiles/KK.in (an s quark
# beside the u quark) and one-derivative displaced operators in all six
# directions on HYP-smeared links; 6 random vectors per flavour, TB16 EI8 DF4.
_KK_OPS = ["g4.d0.p0", "g5.d0.p0", "g5.d>x,<x,>y,<y,>z,<z.p0"]
CONFIGS["cfg5_48x96"] = Workload(
    "cfg5_48x96", Lt=96, L=48, nev=220, n_rnd=12, dilT=16, dilE=8,
    operators=PION_RHO_OPERATORS + _KK_OPS,
    correlators=(["C2c:Q0:Op9:Q0:Op9:P0,1,2,3,4"]
                 + [f"C3c:Q0:Op9:Q0:Op{k}:Q0:Op9:P0,1,2,3,4" for k in range(9)]
                 + ["C4cD:Q0:Op9:Q0:Op9:Q0:Op9:Q0:Op9:P0,1,2,3,4",
                    "C4cB:Q0:Op9:Q0:Op9:Q0:Op9:Q0:Op9:P0,1,2,3,4",
                    "C4cV:Q0:Op9:Q0:Op9:Q0:Op9:Q0:Op9:P0,1,2,3,4",
                    "C2c:Q0:Op11:Q1:Op11", "C4cD:Q0:Op11:Q1:Op11:Q0:Op11:Q1:Op11",
                    "C4cC:Q0:Op11:Q1:Op11:Q0:Op11:Q1:Op11",
                    "C20:Q0:Op10:Q1:Op10", "C40D:Q0:Op10:Q1:Op10:Q0:Op10:Q1:Op10",
                    "C40V:Q0:Op10:Q1:Op10:Q0:Op10:Q1:Op10",
                    "C40C:Q0:Op10:Q1:Op10:Q0:Op10:Q1:Op10",
                    "C40B:Q0:Op10:Q1:Op10:Q0:Op10:Q1:Op10",
                    "C2c:Q0:Op12:Q0:Op12:P0"]),
    quark_lines=("u:6:TB:16:EI:8:DF:4:synthetic", "s:6:TB:16:EI:8:DF:4:synthetic"),
    extra={"alpha1": 0.62, "alpha2": 0.62, "iterations": 3},
    seed=909, orthonormal=False, v_period=8, eigenvector_slots=2, factors_per_block_pair=True,
    description="48^3x96 Nev=220: pipi I=1 + KK + displaced, streamed eigenvectors")


# Uneven batch: six configurations of 24^3 x 48 and 32^3 x 64 with Nev from 64
# to 220, 3-6 random vectors and time dilution 8 or 16, the pion/rho operators
# with |p|^2 <= 1 (instances with 3 random vectors drop the four-point
# diagrams, which need four distinct random indices).
def uneven_instance(i, L, Lt, nev, n_rnd, dilT):
    ops = [o.replace("p0,1,2,3,4", "p0,1") for o in PION_RHO_OPERATORS]
    corr = (["C2c:Q0:Op9:Q0:Op9:P0,1"]
            + [f"C3c:Q0:Op9:Q0:Op{k}:Q0:Op9:P0,1" for k in range(9)])
    if n_rnd >= 4:
        corr += ["C4cD:Q0:Op9:Q0:Op9:Q0:Op9:Q0:Op9:P0,1",
                 "C4cB:Q0:Op9:Q0:Op9:Q0:Op9:Q0:Op9:P0,1",
                 "C4cV:Q0:Op9:Q0:Op9:Q0:Op9:Q0:Op9:P0,1"]
    return Workload(f"cfg4_{i}_{L}x{Lt}_nev{nev}", Lt=Lt, L=L, nev=nev, n_rnd=n_rnd, dilT=dilT,
                    dilE=8, operators=ops, correlators=corr, seed=1000 + i, orthonormal=False,
                    description=f"{L}^3x{Lt} Nev={nev}, {n_rnd} random vectors, TB{dilT}")


UNEVEN_CFG4 = [uneven_instance(i, *a) for i, a in enumerate([
    (24, 48, 64, 3, 8), (24, 48, 96, 4, 16), (24, 48, 120, 5, 8),
    (32, 64, 160, 6, 16), (32, 64, 220, 4, 16), (32, 64, 120, 5, 8)])]
