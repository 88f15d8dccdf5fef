"""GB300-native stochastic series expansion (SSE) update engine.

Host-side mirror of lukas-weber/StochasticSeriesExpansion.jl's model and
Carlo.jl MC interfaces over the C-ABI CUDA library ``libssegpu.so``.
"""

from .util import split_idx, join_idx, worm_action, worm_inverse, worm_count, site_of_leg
from .lattice import Lattice, UnitCell, UnitCells, UCBond, UCSite, neel_vector
from .operators import spin_operators, bosonic_a_operator
from .vertex_data import VertexData, make_vertex_data
from .sse_data import SSEData, SSEBond, SSESite, generate_sites_from_bonds
from .abstract_model import AbstractModel
from .magnet import (
    MagnetModel,
    MagnetizationEstimatorSpec,
    all_magnetization_estimators,
    magnetization_estimator_standard_prefix,
)
from .tables import FlatModel, flatten_model, flatten_sse_data
from .cluster import ClusterBasis, ClusterBases, ClusterModel, lift_twobody_operator, build_cluster_hamiltonians
from . import engine
from .mc import MC, MCContext, BatchMC, TemperingMC
