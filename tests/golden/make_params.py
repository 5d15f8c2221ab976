"""Extract the ff_2.1 force-field arrays used by the synthetic config generator
from the reference checkout into tests/golden/ff21_params.npz.

Run here (where the reference checkout exists); the .npz is committed so the
generator works on hosts without the reference.  Sources:
parameters/ff_2.1/{sidechain.h5,environment.h5,hbond.h5,bb_env.dat,membrane.h5} and
parameters/common/rama_reference.pkl.
"""
import os
import pickle
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "..", "upside2-md_gb300"))
from h5lite import H5File  # noqa: E402

# the reference checkout: $UPSIDE_REFERENCE, else a "reference" directory beside the repository
REF = os.environ.get("UPSIDE_REFERENCE", os.path.join(HERE, "..", "..", "..", "reference"))
P = os.path.join(REF, "parameters")


def main():
    out = {}
    with H5File(os.path.join(P, "ff_2.1", "sidechain.h5")) as f:
        for k in ["restype_order", "rotamer_center_fixed", "rotamer_prob", "rotamer_start_stop_bead",
                  "bead_order", "coverage_interaction", "hydrophobe_placement", "hydrophobe_interaction",
                  "pair_interaction", "restype_and_chi_and_state"]:
            out["sc_" + k] = f.read("/" + k)
    with H5File(os.path.join(P, "ff_2.1", "environment.h5")) as f:
        for k in ["restype_order", "weights", "coverage_param", "energies", "scale", "center", "sharpness"]:
            out["env_" + k] = f.read("/" + k)
        out["env_energies_offset"] = np.float64(f.attr("/energies", "offset"))
        out["env_energies_inv_dx"] = np.float64(f.attr("/energies", "inv_dx"))
    with H5File(os.path.join(P, "ff_2.1", "hbond.h5")) as f:
        out["hbond_parameter"] = f.read("/parameter")
    out["bb_env"] = np.loadtxt(os.path.join(P, "ff_2.1", "bb_env.dat"))
    with H5File(os.path.join(P, "ff_2.1", "membrane.h5")) as f:
        for k in ["names", "cb_energy", "hb_energy", "icb_energy", "ihb_energy", "burial_nodes"]:
            out["mem_" + k] = f.read("/" + k)
        for k in ["cb_z_min", "cb_z_max", "hb_z_min", "hb_z_max"]:
            out["mem_" + k] = np.float64(f.attr("/", k))
    with open(os.path.join(P, "common", "rama_reference.pkl"), "rb") as fh:
        out["rama_reference"] = np.asarray(pickle.load(fh, encoding="latin1"), dtype=np.float64)
    np.savez_compressed(os.path.join(HERE, "ff21_params.npz"), **out)


if __name__ == "__main__":
    main()
