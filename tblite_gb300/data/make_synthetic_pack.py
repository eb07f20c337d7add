"""Write the synthetic element-data pack ``element_data_synthetic.json``.

GFN2-xTB and GFN1-xTB take part of their element data from libraries that are not part of the
reference tree (mctc-lib: covalent radii, Pauling electronegativities, atomic radii and the
coordination-number counting constants; dftd4 / s-dftd3: the dispersion models' reference
coordination numbers, charges, polarisability-derived C6 coefficients and model constants).  The
engine reads them from an element-data pack whose format holds what those libraries provide:

* ``cn``: counting constants of the double-exponential coordination number and covalent radii;
* ``pauling_en``, ``atomic_rad``: per element;
* ``d4``: model constants (charge scaling ``ga``, ``gc``, weighting ``wf``, CN counting
  ``cn_kn``, ``cn_k4..6``, cutoffs, ATM ``atm_alpha``, smooth-cutoff widths ``width2``,
  ``width3``) and per element the reference CNs, reference charges, Gaussian-weight counts,
  effective charges, hardnesses, <r4>/<r2> ratios, covalent radii and electronegativities;
  ``c6`` holds the reference C6 coefficients per element PAIR, ``"Za-Zb"`` (Za <= Zb) -> a
  nref(Za) x nref(Zb) matrix, the layout of dftd4's c6(iref, jref, izp, jzp) table;
* ``cn_exp``, ``d3``: the exponential counting constant of GFN1-xTB and the D3 constants.

EVERY number written by this script is an arbitrary synthetic value chosen only so that the
kernels and the CPU oracle can be compared on the same inputs: none is taken from mctc-lib,
dftd4 or s-dftd3, and total energies computed with this pack are not comparable with the
reference's.  The C6 pair matrices are synthesised as geometric means of arbitrary per-reference
strengths (a convenience of this script, not part of the format).

Usage: ``python tblite_gb300/data/make_synthetic_pack.py`` (then ``gen_element_data.py``).
"""
import json
import math
from pathlib import Path

HERE = Path(__file__).resolve().parent
ELEMENTS = [1, 6, 7, 8]


def main():
    per = {  # arbitrary synthetic per-element values
        "rcov": {1: 0.75, 6: 1.85, 7: 1.75, 8: 1.65},
        "en": {1: 2.1, 6: 2.6, 7: 3.0, 8: 3.5},
        "rad": {1: 0.62, 6: 1.42, 7: 1.40, 8: 1.36},
        "gam": {1: 0.45, 6: 0.40, 7: 0.45, 8: 0.50},
        "r4r2": {1: 2.0, 6: 3.1, 7: 2.7, 8: 2.4},
        "refcn": {1: [0.0, 1.0], 6: [0.0, 2.0, 4.0], 7: [0.0, 2.0, 3.0], 8: [0.0, 2.0]},
        "strength": {1: [6.5, 3.1], 6: [46.0, 37.0, 25.0], 7: [24.0, 20.0, 18.0],
                     8: [15.5, 12.0]},
    }
    arbitrary = "arbitrary synthetic value (not from mctc-lib, dftd4 or s-dftd3)"
    c6 = {}
    for a in ELEMENTS:
        for b in ELEMENTS:
            if a <= b:
                c6[f"{a}-{b}"] = [[math.sqrt(x * y) for y in per["strength"][b]]
                                  for x in per["strength"][a]]
    pack = {
        "name": "synthetic-v2",
        "provenance": "SYNTHETIC stand-in values chosen for kernel-vs-oracle parity only: every "
                      "number is " + arbitrary + "; total energies computed with this pack are "
                      "not comparable with the reference.  Written by make_synthetic_pack.py.",
        "elements": ELEMENTS,
        "cn": {"provenance": arbitrary, "kind": "dexp", "ka": 9.0, "kb": 18.0, "rshift": 1.5,
               "cutoff": 25.0, "rcov": {str(z): per["rcov"][z] for z in ELEMENTS}},
        "pauling_en": {str(z): per["en"][z] for z in ELEMENTS},
        "atomic_rad": {str(z): per["rad"][z] for z in ELEMENTS},
        "d4": {"provenance": arbitrary, "ga": 2.8, "gc": 2.2, "wf": 5.5, "cn_kn": 7.0,
               "cn_k4": 4.0, "cn_k5": 19.0, "cn_k6": 250.0, "cn_cutoff": 25.0,
               "disp2_cutoff": 50.0, "disp3_cutoff": 25.0, "atm_alpha": 14.0,
               "width2": 0.0, "width3": 0.0,
               "rcov": {str(z): per["rcov"][z] for z in ELEMENTS},
               "en": {str(z): per["en"][z] for z in ELEMENTS},
               "zeff": {str(z): float(z) for z in ELEMENTS},
               "gam": {str(z): per["gam"][z] for z in ELEMENTS},
               "r4r2": {str(z): per["r4r2"][z] for z in ELEMENTS},
               "refcn": {str(z): per["refcn"][z] for z in ELEMENTS},
               "refq": {str(z): [0.0] * len(per["refcn"][z]) for z in ELEMENTS},
               "ngw": {str(z): [1] * len(per["refcn"][z]) for z in ELEMENTS},
               "c6": c6},
        "cn_exp": {"provenance": arbitrary, "kind": "exp counting function 1/(1+exp(-k (r0/r - "
                   "1))), r0 = rcov_A + rcov_B with the rcov of the cn block (GFN1 self-energy "
                   "shift)", "k": 15.0, "cutoff": 25.0},
        "d3": {"provenance": arbitrary, "kind": "D3(BJ) two-body model of GFN1: coordination "
               "numbers with the exp counting function (k1) over the d4 block's rcov; Gaussian "
               "weights exp(-k3 (CN - CNref)^2) over the d4 block's reference CNs; C6 from the "
               "d4 block's pair table; C8 = 3 C6 sqrt(Q_A Q_B), Q = r4r2 of the d4 block",
               "k1": 15.0, "k3": 3.5, "cn_cutoff": 25.0, "disp2_cutoff": 50.0},
    }
    (HERE / "element_data_synthetic.json").write_text(json.dumps(pack, indent=1) + "\n")
    print("wrote element_data_synthetic.json")


if __name__ == "__main__":
    main()
