"""Full-size oracle reference for the 60,000-site Wang-AL chain system (test fixture).

    python tests/golden/make_c60k_reference.py      # a few minutes on 8 cores

Runs the CPU oracle (reference CG, tolerance 1e-10, direct matrix-vector
product) on the precision benchmark geometry (150 self-avoiding chains of 200
sites in 10,000 waters, Wang-AL linear Thole damping, 1-2/1-3 exclusions,
synth.chain_system(seed=3)) with the point-charge field of seed 7, and stores
in tests/golden/c60k_seed7.npz: the polarization energy, the residual history
and product count, the 2-norm and the sum of the dipoles, and the dipoles and
the permanent-multipole field of 3,000 sampled sites (indices included).  The
GPU suite compares fresh GPU solves against it.
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from openmmpol_gb300 import synth  # noqa: E402
from oracle.oracle import OracleSystem  # noqa: E402

GEOM_SEED, FIELD_SEED, N_SAMPLE = 3, 7, 3000


def main(out=os.path.join(HERE, "c60k_seed7.npz")):
    import tempfile
    c = synth.chain_system(seed=GEOM_SEED)
    with tempfile.TemporaryDirectory() as d:
        path = synth.write_mmp(os.path.join(d, "c60k.mmp"), c)
        o = OracleSystem(path)
        o.set_tol(1e-10)
        cmm = o.cmm
        ef, _, _ = synth.point_charge_field(cmm[o.polar_mm], c.box_center(), seed=FIELD_SEED,
                                            all_sites_bohr=cmm)
        t = time.time()
        e_m2d = o.e_m2d()
        o.set_external_field(ef)
        dt = time.time() - t
        ipd = o.ipd
        ep = o.get_polelec_energy()
        idx = np.sort(np.random.default_rng(7).choice(o.pol_atoms, N_SAMPLE, replace=False))
        np.savez_compressed(out, energy=ep, hist=o.residual_history(0), iters=np.array([o.last_iterations(0)]),
                            matvecs=o.matvec_count(), norm=np.linalg.norm(ipd), sum=ipd.sum(), idx=idx,
                            ipd_sample=ipd[:, idx, :], e_m2d_sample=e_m2d[:, idx, :], pol_atoms=o.pol_atoms,
                            seconds=dt)
    print("wrote", out, "energy", ep, "in %.0f s" % dt)


if __name__ == "__main__":
    main()
