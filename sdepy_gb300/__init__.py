"""sdepy_gb300: sdepy's Monte Carlo path-integration hot path on one GB300.

Drop-in process classes (same names, keywords and results as sdepy's
presets) integrate on the GPU through the C-ABI of include/sdepy_gb300.h;
``montecarlo`` summarises samples with device reductions.
"""
from .infrastructure import (
    process, philox_rng, wiener_source, poisson_source, cpoisson_source,
    norm_rv, uniform_rv, exp_rv, double_exp_rv, odd_wiener_source,
    even_poisson_source, even_cpoisson_source)
from .integration import (
    wiener_process, lognorm_process, ornstein_uhlenbeck_process,
    hull_white_process, hull_white_1factor_process, full_heston_process,
    heston_process, jumpdiff_process, merton_jumpdiff_process,
    kou_jumpdiff_process, cox_ingersoll_ross_process)
from .usersde import integrate
from . import infrastructure
from .montecarlo import montecarlo   # the class, as sdepy exports it

__version__ = '0.1.0'

__all__ = [
    'process', 'philox_rng', 'wiener_source', 'poisson_source',
    'cpoisson_source', 'norm_rv', 'uniform_rv', 'exp_rv', 'double_exp_rv',
    'odd_wiener_source', 'even_poisson_source', 'even_cpoisson_source',
    'wiener_process', 'lognorm_process', 'ornstein_uhlenbeck_process',
    'hull_white_process', 'hull_white_1factor_process',
    'full_heston_process', 'heston_process', 'jumpdiff_process',
    'merton_jumpdiff_process', 'kou_jumpdiff_process',
    'cox_ingersoll_ross_process', 'integrate', 'montecarlo',
]
