"""flare_gb300: GB300-native (sm_103a) sparse-GP prediction for FLARE's
B2 / NormalizedDotProduct / SparseGP / SGP_Calculator path."""
from .core import (B2, ClusterDescriptor, DescriptorValues,  # noqa: F401
                   NormalizedDotProduct, SparseGP, Structure, get_precision,
                   set_precision)
from .sparse_gp import SGP_Wrapper  # noqa: E402,F401
from .calculator import SGP_Calculator  # noqa: E402,F401
