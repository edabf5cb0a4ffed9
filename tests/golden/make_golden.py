"""Regenerate tests/golden/loglik_golden.json from the reference's own known-answer CSVs.

The reference ships LL / dLL/dtheta known answers (and, for data1-scal, the leave-one-out value and its
gradient, binding_consistency_test.py:46-72) for a gauss kernel at theta = 0.3 * ones(d), constant
trend, no normalisation, NoiseModel None (bindings/Python/pylibkriging/tests/binding_consistency_test.py:46-121
reads them from tests/references/). This script copies the inputs and answers verbatim (every CSV value
parsed to float64) into one JSON fixture so that the tests can run where the reference tree is absent.

Usage:  python tests/golden/make_golden.py path/to/libKriging-source-tree
"""
import json
import sys
from pathlib import Path

import numpy as np


def _csv(path):
    return np.atleast_1d(np.genfromtxt(path, delimiter=","))


def main(ref_root):
    refs = Path(ref_root) / "tests" / "references"
    cases = []
    for i in range(1, 11):
        prefix = f"data2-grad-{i}"
        X = np.atleast_2d(np.genfromtxt(refs / f"{prefix}-X.csv", delimiter=","))
        cases.append(dict(
            name=prefix,
            X=X.tolist(),
            y=_csv(refs / f"{prefix}-y.csv").tolist(),
            ll=float(_csv(refs / f"{prefix}-result-logLikelihood.csv")[0]),
            grad=_csv(refs / f"{prefix}-result-logLikelihoodGrad.csv").tolist(),
        ))
    prefix = "data1-scal"
    X = _csv(refs / f"{prefix}-X.csv").reshape(-1, 1)
    cases.append(dict(
        name=prefix,
        X=X.tolist(),
        y=_csv(refs / f"{prefix}-y.csv").tolist(),
        ll=float(_csv(refs / f"{prefix}-result-logLikelihood.csv")[0]),
        grad=_csv(refs / f"{prefix}-result-logLikelihoodGrad.csv").tolist(),
        loo=float(_csv(refs / f"{prefix}-result-leaveOneOut.csv")[0]),
        loo_grad=_csv(refs / f"{prefix}-result-leaveOneOutGrad.csv").tolist(),
    ))
    out = dict(
        source="libKriging tests/references/{data2-grad-1..10,data1-scal}-*.csv",
        kernel="gauss", theta_value=0.3, regmodel="constant", normalize=False, noise_model="none",
        tolerance_relative=1e-12,
        cases=cases,
    )
    dst = Path(__file__).with_name("loglik_golden.json")
    dst.write_text(json.dumps(out, indent=1))
    print(f"wrote {dst} ({len(cases)} cases)")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py path/to/libKriging-source-tree")
    main(sys.argv[1])
