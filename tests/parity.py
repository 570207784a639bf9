"""The parity rules (oracle/parity.py), under the name the tests import."""
from oracle.parity import (TOL_ULP, _same_float, check, compare, exact_vs_leaf_only,  # noqa: F401
                           tree_dependent_rays, tri_box_pass)
