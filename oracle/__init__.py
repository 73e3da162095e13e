"""Test infrastructure only: a CPU restatement of gplite's GP hot path.

This package is the oracle that the CUDA library is checked against. Only
``tests/``, ``__graft_entry__.smoke()`` and the ``cpu_baseline`` / reference arm
of ``bench.py`` may import it, and only as the checker or as the timed CPU
baseline. The product package ``gplite_gb300`` never imports it.

Parity status: the reference (R package gplite 0.13.0) cannot run here (no R
interpreter, no Rcpp/RcppArmadillo headers), and it ships no golden vectors.
The restatement is pinned against the reference's own known-answer tests
(closed-form Gaussian marginal likelihood and predictive equations of
tests/testthat/test_basic.R:64-132, normalisation invariance of
tests/testthat/test_normalization.R:81-141, parameter round trip of
tests/testthat/test_param.R:73-85), restated in ``tests/test_oracle.py`` with
tighter tolerances, plus identities that follow from the formulas. Values the
reference's tests do not pin (Laplace/EP/FITC evidences, LOO values) are
pinned only by the line-by-line restatement: parity partially unpinned.
"""
from . import gplite_ref  # noqa: F401
