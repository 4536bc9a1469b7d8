"""Generate tests/golden/l4/* from the reference's L4 integration test.

Source (reference tree, read-only): tests/integration-L4/
  test_all.ini                          infile (4^4 lattice, Nev=16, u+s quarks,
                                        5 random vectors each, TB:2 EI:2 DF:4)
  eigensystem/eigenvectors.1000.00t     LapH eigenvectors, t = 0..3
  {light,strange}/cnfg1000/rnd_vec_0r/  perambulators and Z2 noise
  correlators-reference/*.h5            goldens, compared by
                                        tests/integration-L4/compare:16 with
                                        h5diff -r -d 1e-12

Outputs (committed):
  l4/test_all.ini        the infile, verbatim
  l4/inputs.npz          V [Lt][nev][dim_row] (each timeslice column-major),
                         peram [n_rnd][cols][rows] (column-major after the
                         reference re-sort, src/Perambulator.cpp:53-64),
                         noise [n_rnd][Lt*4*nev], and the raw bytes of one
                         file of each kind for the reader tests
  l4/goldens.npz         names, diagram of each name, values [n][Lt] complex
  l4/gauge_conf.1000     gauge/conf.1000 verbatim: a LIME/ILDG double-precision
                         4^4 gauge field whose xlf-info record states its
                         average plaquette (the reader's known answer)

The re-sort is done here with numpy, independently of the oracle and engine
readers, so the three implementations check each other.

Run:  python tests/golden/make_l4_fixtures.py [/path/to/reference] [--only gauge]
"""
from __future__ import annotations

import os
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent))
import h5lite  # noqa: E402

Lt, L, NEV = 4, 4, 16
DIM_ROW = 3 * L ** 3
DIL_T, DIL_E, DIL_D = 2, 2, 4
QUARKS = [("u", "light"), ("s", "strange")]
N_RND_PER_QUARK = 5


def peram_name(q, r):
    return (f"perambulator.rndvecnb{r:02d}.{q}.TsoB{Lt // DIL_T:04d}.VsoI{DIL_E:04d}.DsoF{DIL_D}"
            f".TsiF{Lt:04d}.SsiF{L ** 3:04d}.DsiF4.CsiF3.smeared0.01000")


def resort_perambulator(raw: np.ndarray) -> np.ndarray:
    """File order [t1][ev1][d1] x [b][ev2][d2] -> matrix rows (t1, d1, ev1),
    columns (b, d2, ev2), returned as [cols][rows] (column-major storage)."""
    nb = Lt // DIL_T
    a = raw.reshape(Lt, NEV, 4, nb, DIL_E, DIL_D)
    m = a.transpose(0, 2, 1, 3, 5, 4).reshape(4 * NEV * Lt, nb * DIL_D * DIL_E)
    return np.ascontiguousarray(m.T)


def write_gauge(ref_root: Path):
    base = ref_root / "tests" / "integration-L4"
    (HERE / "l4" / "gauge_conf.1000").write_bytes((base / "gauge" / "conf.1000").read_bytes())


def main(ref_root: Path):
    base = ref_root / "tests" / "integration-L4"
    out = HERE / "l4"
    out.mkdir(exist_ok=True)
    write_gauge(ref_root)
    (out / "test_all.ini").write_text((base / "test_all.ini").read_text())

    V = np.zeros((Lt, NEV, DIM_ROW), np.complex128)
    for t in range(Lt):
        raw = np.fromfile(base / "eigensystem" / f"eigenvectors.1000.{t:03d}", dtype="<c16")
        assert raw.size == DIM_ROW * NEV
        V[t] = raw.reshape(NEV, DIM_ROW)
    perams, noises = [], []
    raw_peram = raw_noise = None
    for q, path in QUARKS:
        for r in range(N_RND_PER_QUARK):
            d = base / path / "cnfg1000" / f"rnd_vec_{r:02d}"
            rp = np.fromfile(d / peram_name(q, r), dtype="<c16")
            assert rp.size == 4 * NEV * Lt * (Lt // DIL_T) * DIL_E * DIL_D
            perams.append(resort_perambulator(rp))
            rn = np.fromfile(d / f"randomvector.rndvecnb{r:02d}.{q}.nbev{NEV:04d}.1000", dtype="<c16")
            assert rn.size == Lt * 4 * NEV
            noises.append(rn)
            if raw_peram is None:
                raw_peram = (d / peram_name(q, r)).read_bytes()
                raw_noise = (d / f"randomvector.rndvecnb{r:02d}.{q}.nbev{NEV:04d}.1000").read_bytes()
    raw_eig = (base / "eigensystem" / "eigenvectors.1000.000").read_bytes()
    np.savez_compressed(
        out / "inputs.npz", V=V, peram=np.stack(perams), noise=np.stack(noises),
        raw_eig=np.frombuffer(raw_eig, np.uint8), raw_peram=np.frombuffer(raw_peram, np.uint8),
        raw_noise=np.frombuffer(raw_noise, np.uint8),
        dims=np.array([Lt, L, L, L, NEV, DIL_T, DIL_E, 2 * N_RND_PER_QUARK]))

    names, diags, vals = [], [], []
    for f in sorted((base / "correlators-reference").glob("*.h5")):
        diag = f.name.split("_cnfg")[0]
        for name, v in sorted(h5lite.read_correlators(f).items()):
            names.append(name)
            diags.append(diag)
            vals.append(v)
    np.savez_compressed(out / "goldens.npz", names=np.array(names), diagrams=np.array(diags),
                        values=np.stack(vals))
    # Dilution-iterator golden text (tests/dilution-iterator/control.txt, the
    # output of main/test-iterator.cpp), verbatim.
    ctl = ref_root / "tests" / "dilution-iterator" / "control.txt"
    (HERE / "dilution_control.txt").write_text(ctl.read_text())
    print(f"wrote {out}: {len(names)} golden datasets")


if __name__ == "__main__":
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    # the reference tree: first argument, else $SLAPH_REFERENCE_DIR, else a
    # directory named "reference" beside this repository's root
    root = Path(args[0] if args else os.environ.get(
        "SLAPH_REFERENCE_DIR", str(Path(__file__).resolve().parents[3] / "reference")))
    if "--only" in sys.argv and sys.argv[sys.argv.index("--only") + 1] == "gauge":
        write_gauge(root)
    else:
        main(root)
