"""Full-size oracle reference for the 90,000-site water box (test fixture).

    python tests/golden/make_w30k_reference.py      # ~7 min on 8 cores

Runs the CPU oracle (reference CG, tolerance 1e-10, direct matrix-vector
product) on the benchmark geometry (30,000 AMOEBA waters, seed 1) with the
point-charge field of seed 103, and stores in tests/golden/w30k_seed103.npz:
the polarization energy, the residual history and product count, the 2-norm
and the sum of each dipole set, and the dipoles of 3,000 sampled sites
(indices included).  The GPU suite compares a fresh GPU solve against it.
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from openmmpol_gb300 import synth  # noqa: E402
from oracle.oracle import OracleSystem  # noqa: E402

N_WATERS, GEOM_SEED, FIELD_SEED, N_SAMPLE = 30000, 1, 103, 3000


def main(out=os.path.join(HERE, "w30k_seed103.npz")):
    import tempfile
    w = synth.water_cluster(N_WATERS, seed=GEOM_SEED)
    with tempfile.TemporaryDirectory() as d:
        path = synth.write_mmp(os.path.join(d, "w30k.mmp"), w)
        o = OracleSystem(path)
        o.set_tol(1e-10)
        cmm = o.cmm
        ef, _, _ = synth.point_charge_field(cmm[o.polar_mm], w.box_center(), seed=FIELD_SEED,
                                            all_sites_bohr=cmm)
        t = time.time()
        o.set_external_field(ef)
        dt = time.time() - t
        ipd = o.ipd
        ep = o.get_polelec_energy()
        idx = np.sort(np.random.default_rng(7).choice(o.pol_atoms, N_SAMPLE, replace=False))
        np.savez_compressed(out, energy=ep, hist_d=o.residual_history(0), hist_p=o.residual_history(1),
                            iters=np.array([o.last_iterations(0), o.last_iterations(1)]),
                            matvecs=o.matvec_count(), norms=np.linalg.norm(ipd.reshape(2, -1), axis=1),
                            sums=ipd.reshape(2, -1).sum(axis=1), idx=idx, ipd_sample=ipd[:, idx, :],
                            seconds=dt)
    print("wrote", out, "energy", ep, "in %.0f s" % dt)


if __name__ == "__main__":
    main()
