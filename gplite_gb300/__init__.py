"""gplite_gb300: gplite's GP hot path (fit / energy / gradient / pred / LOO)
on one GB300 GPU through the libgpgp C ABI (include/gpgp.h)."""
from .objects import (approx_ep, approx_laplace, cf_const, cf_lin, cf_matern32, cf_matern52,  # noqa: F401
                      cf_nn, cf_periodic, cf_prod, cf_sexp, lik_bernoulli, lik_betabinom,
                      lik_binomial, lik_gaussian, lik_poisson, method_fitc, method_full, method_rbf, method_rf,
                      prior_fixed, prior_half_t, prior_logunif, prior_lognormal)
from .gp import (GP, eval_cf, get_param, gp_compare, gp_draw, gp_energy, gp_energy_grad, gp_fit,  # noqa: F401
                 gp_init, gp_loo, gp_optim, gp_pred, gp_pred_cov, set_param, model_field)

__version__ = "0.1.0"
