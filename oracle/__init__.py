"""CPU oracles for the visibility simulator and the median filter (test
infrastructure only; see ``oracle/vis_oracle.py`` and
``oracle/median_oracle.py``).  Never imported by the product package."""
from .vis_oracle import (SPEED_OF_LIGHT, bilinear_beam, phasors,  # noqa: F401
                         hermitian_product, vis_oracle, vis_oracle_partial,
                         rel_frobenius)
from .median_oracle import median_filter_oracle  # noqa: F401
