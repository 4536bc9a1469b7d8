"""The reference's `contract` executable on the engine (main/contract.cpp:55-105).

    python -m slaph_gb300 -i <infile> [--start_config N ...] [--precision mixed|fp64]
                          [--accumulator native|kahan]

Reads the infile (with the reference's command-line overrides), then for every
configuration start_config..end_config in steps of delta_config: reads the
perambulators and random vectors of its file names (build_IO_names), creates
the VdaggerV operators as handling_vdaggerv asks (from the eigenvector files,
with the gauge field and HYP smearing when displaced operators need it, or from
VdaggerV files), contracts, and writes one HDF5 file per diagram to
output_path.  The same files and datasets as the reference's.
"""
from __future__ import annotations

import argparse
import os
import sys
import time

from . import GlobalData
from ._lib import SlaphError
from .engine import FP64, KAHAN, MIXED, NATIVE, Engine, OperatorFactory, contract, write_diagrams
from .frontend import read_eigenvectors, read_gauge_lime, read_perambulator, read_random_vector


def run_configuration(gd: GlobalData, eng: Engine, fac: OperatorFactory, config: int,
                      precision: int, accumulator: int) -> dict:
    d = gd.dims
    dim_row = 3 * d.Lx * d.Ly * d.Lz
    # Perambulator::read_perambulators_from_separate_files and
    # RandomVector::read_random_vectors_from_separate_files (main/contract.cpp:89-92)
    for r in range(d.n_rnd):
        eng.set_perambulator(r, read_perambulator(gd.io_name(config, 1, r), d.Lt, d.nev,
                                                  d.dilT, d.dilE, 4))
        eng.set_random_vector(r, read_random_vector(gd.io_name(config, 2, r),
                                                    d.Lt * 4 * d.nev))
    # OperatorFactory::create_operators (src/OperatorFactory.cpp:507-520)
    if gd.get_str("handling_vdaggerv") in ("build", "write"):
        prefix = gd.io_name(config, 0)
        for t in range(d.Lt):
            eng.set_eigenvectors(t, read_eigenvectors(f"{prefix}{t:03d}", dim_row, d.nev))
        if gd.plan.need_gaugefield:
            U = read_gauge_lime(gd.io_name(config, 4), d.Lt, d.Lx, d.Ly, d.Lz, 3)
            fac.set_gauge_field(U)
    fac.create_operators(precision, config=config)
    corr = contract(eng, gd, precision, accumulator,
                    gd.get_int("single_time_slice_combination"))
    write_diagrams(gd.get_str("output_path"), corr, gd.io_name(config, 3))
    return corr


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(prog="python -m slaph_gb300",
                                 description="sLapH contractions on the GB300 engine")
    ap.add_argument("-i", "--input", default="LapHs.in", help="infile (default LapHs.in)")
    ap.add_argument("--precision", choices=["mixed", "fp64"], default="mixed")
    ap.add_argument("--accumulator", choices=["native", "kahan"], default="native")
    args, overrides = ap.parse_known_args(argv)
    try:
        gd = GlobalData.from_infile(args.input, overrides)
    except SlaphError as e:
        print(e, file=sys.stderr)
        return 1
    start, end = gd.get_int("start_config"), gd.get_int("end_config")
    delta = gd.get_int("delta_config")
    if delta <= 0:
        print("The 'delta_config' option has been set to a non-positive value. This makes "
              "no sense.", file=sys.stderr)
        return 1
    precision = MIXED if args.precision == "mixed" else FP64
    accumulator = KAHAN if args.accumulator == "kahan" else NATIVE
    eng = Engine(gd.dims)
    fac = OperatorFactory(eng, gd)
    for config in range(start, end + 1, delta):
        print(f"\nprocessing configuration: {config}\n", flush=True)
        t0 = time.time()
        try:
            corr = run_configuration(gd, eng, fac, config, precision, accumulator)
        except SlaphError as e:
            print(e, file=sys.stderr)
            return 1
        n = sum(len(ds) for ds in corr.values())
        print(f"\t{n} correlators of {len(corr)} diagrams written to "
              f"{os.path.join(gd.get_str('output_path'), '*' + gd.io_name(config, 3))} "
              f"in {time.time() - t0:.2f} s", flush=True)
    eng.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
