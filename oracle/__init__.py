"""CPU oracles for the visibility simulator, the median filter and the
Omnical solver (test infrastructure only; see ``oracle/vis_oracle.py``,
``oracle/median_oracle.py`` and ``oracle/omnical_oracle.py``).  Never
imported by the product package."""
from .vis_oracle import (SPEED_OF_LIGHT, bilinear_beam, phasors,  # noqa: F401
                         hermitian_product, vis_oracle, vis_oracle_partial,
                         rel_frobenius)
from .median_oracle import median_filter_oracle  # noqa: F401
from .omnical_oracle import omnical_oracle, redundant_problem  # noqa: F401
