"""Make the FP64 reference fixture of the 1000 x 1000 x 1000, R = 32 headline solve.

The tensor is the seeded host draw of ``datagen.make_cpd_problem_host`` (U[0,1] factors with
equalised column norms, seed 2; 30 dB Gaussian noise; initial factors U[0,1], seed 3), which
gives the same values on every machine.  The FP64 OpenMP restatement of the reference's ALS
driver (oracle/cpd_omp.c, include/CpdOpenMP.hpp:266-329) runs on it under the reference's
own stopping rule with its default options (include/PARTENSOR_basic.hpp:187-196:
threshold_error 1e-3, max_iter 20, Nesterov tolerance 1e-2, acceleration and normalisation
on): stop when rel < 1e-3 or after 20 sweeps (include/Cpd.hpp:339).  Saved (npz):

  rel_fp64            the relative fit error of the FP64 solve when it stops
  trace               per sweep: f_value, rel_costFunction, acceleration accepted
  factors             the final factors (float32, I_k x R), for the congruence check
  frob, noise_rel     ||X||^2 and ||noise|| / ||X|| of the draw (a fingerprint of the data)
  probe_idx, probe    a few tensor entries (a second fingerprint)
  long_trace          with --long N: the rel trace of an N-sweep run of the same solve, which
                      shows how far the 20-sweep fit is from the converged one

Run from the repository root:  python tests/golden/make_headline_fp64.py [--long 60]
"""
from __future__ import annotations

import argparse
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "headline_1000cubed_r32_fp64.npz")
DIMS, RANK, SEED, INIT_SEED, SNR_DB = [1000, 1000, 1000], 32, 2, 3, 30.0
PROBE_IDX = np.array([0, 1, 999, 1000, 123456789, 500000000, 999999999], dtype=np.int64)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--long", type=int, default=0, help="also run this many sweeps (convergence check)")
    ap.add_argument("--threads", type=int, default=0)
    args = ap.parse_args()
    import __graft_entry__ as ge
    ge.load_package()
    from partensor_toolbox_gb300 import datagen as dg
    from oracle import omp
    t = time.time()
    p = dg.make_cpd_problem_host(DIMS, RANK, seed=SEED, init_seed=INIT_SEED, snr_db=SNR_DB,
                                 equalize_columns=True)
    print(f"data {time.time() - t:.1f} s  noise_rel {p.noise_rel:.9f}  frob {p.frob:.9e}", flush=True)
    t = time.time()
    fs, st, tr = omp.cpd_als(p.X, DIMS, RANK, p.init_factors, threshold_error=1e-3, max_iter=20,
                             nthreads=args.threads)
    secs = time.time() - t
    print(f"fp64 solve {secs:.1f} s, {st.ao_iter} sweeps, rel {st.rel_costFunction:.9f}", flush=True)
    extra = {}
    if args.long:
        t = time.time()
        _, st_l, tr_l = omp.cpd_als(p.X, DIMS, RANK, p.init_factors, threshold_error=1e-3,
                                    max_iter=args.long, nthreads=args.threads)
        print(f"long solve {time.time() - t:.1f} s, rel {st_l.rel_costFunction:.9f}", flush=True)
        extra["long_trace"] = tr_l
    np.savez_compressed(OUT, dims=np.array(DIMS), rank=RANK, seed=SEED, init_seed=INIT_SEED, snr_db=SNR_DB,
                        rel_fp64=st.rel_costFunction, f_value=st.f_value, ao_iter=st.ao_iter,
                        accel_coeff=st.accel_coeff, accel_fail=st.accel_fail, trace=tr,
                        factors=np.stack([f.astype(np.float32) for f in fs]), frob=p.frob,
                        noise_rel=p.noise_rel, probe_idx=PROBE_IDX, probe=p.X[PROBE_IDX],
                        seconds=secs, threads=args.threads or (os.cpu_count() or 1), **extra)
    print("wrote", OUT)


if __name__ == "__main__":
    main()
