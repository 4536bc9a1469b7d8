"""Input files in the reference's formats and names, for running the engine's
command line the way the reference's `contract` runs (test helper)."""
import os

import numpy as np


def perambulator_file_bytes(P, Lt, nev, dilT, dilE, dilD=4):
    """The file of a re-sorted perambulator P (complex (cols, rows), the layout
    slaph_read_perambulator returns): rows (t, ev, dirac) and columns (block,
    ev, dirac), dirac fastest, row-major (the inverse of the re-sort of
    src/Perambulator.cpp:53-64)."""
    rows, nb = 4 * nev * Lt, Lt // dilT
    cols = nb * dilE * dilD
    t, ev, d = np.meshgrid(np.arange(Lt), np.arange(nev), np.arange(4), indexing="ij")
    row_file = (4 * nev * t + 4 * ev + d).ravel()
    row = (4 * nev * t + nev * d + ev).ravel()
    b, e2, d2 = np.meshgrid(np.arange(nb), np.arange(dilE), np.arange(dilD), indexing="ij")
    col_file = (dilD * dilE * b + dilD * e2 + d2).ravel()
    col = (dilE * dilD * b + dilE * d2 + e2).ravel()
    M = np.asarray(P).T  # (rows, cols)
    F = np.empty((rows, cols), np.complex128)
    F[np.ix_(row_file, col_file)] = M[np.ix_(row, col)]
    return F.tobytes()


def write_inputs(gd, config, V, peram, noise, root):
    """Eigenvector, perambulator and random-vector files of one configuration
    under root, at the names build_IO_names gives for the infile."""
    d = gd.dims

    def put(name, data):
        path = os.path.join(root, name)
        os.makedirs(os.path.dirname(path), exist_ok=True)
        with open(path, "wb") as f:
            f.write(data)

    prefix = gd.io_name(config, 0)
    for t in range(d.Lt):
        put(f"{prefix}{t:03d}", np.ascontiguousarray(V[t]).tobytes())
    for r in range(d.n_rnd):
        put(gd.io_name(config, 1, r),
            perambulator_file_bytes(peram[r], d.Lt, d.nev, d.dilT, d.dilE))
        put(gd.io_name(config, 2, r), np.ascontiguousarray(noise[r]).tobytes())
