"""Turn the reference's golden HDF5 dumps into small committed fixtures.

Reads test/expected/f1main_expected_{electrons,field,integrated}.h5 from the
reference checkout (the 2-rank end-to-end test, testMPIIntegration.pf:25-142)
and writes tests/golden/f1main_expected.npz.  Run once in a checkout that has
the reference; the GPU machines only see the .npz.

    python tests/golden/make_golden.py /path/to/puffin-reference
"""
import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
import h5mini  # noqa: E402

ATTRS = ("rho", "aw", "eta", "gamma_r", "kappa", "sLengthOfElmZ2", "sStepSize",
         "nSteps", "nZ2", "zbarTotal", "npk_bar", "transArea", "fieldMesh")
INTEGRATED = ("power", "bunchingFundamental", "meanGamma", "beamCurrent")


def main(ref_root):
    exp = os.path.join(ref_root, "test", "expected")
    out = {}
    h = h5mini.H5File(os.path.join(exp, "f1main_expected_electrons.h5"))
    out["electrons"] = h.dataset(h.group_members(h.root())["electrons"])
    h = h5mini.H5File(os.path.join(exp, "f1main_expected_field.h5"))
    members = h.group_members(h.root())
    out["aperp"] = h.dataset(members["aperp"])
    run = h.attributes(members["runInfo"])
    for k in ATTRS:
        out["attr_" + k] = np.array(run[k])
    h = h5mini.H5File(os.path.join(exp, "f1main_expected_integrated.h5"))
    members = h.group_members(h.root())
    for k in INTEGRATED:
        if k in members:
            out["int_" + k] = h.dataset(members[k])
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "f1main_expected.npz")
    np.savez_compressed(dst, **out)
    print("wrote", dst, {k: np.shape(v) for k, v in out.items()})


if __name__ == "__main__":
    # the reference project's checkout: first argument or PUFFIN_REFERENCE
    src = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("PUFFIN_REFERENCE")
    if not src:
        sys.exit("usage: make_golden.py <reference checkout> (or set PUFFIN_REFERENCE)")
    main(src)
