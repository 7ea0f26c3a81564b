"""GB300-native Fast-Higashi fit hot path.

Drop-in modules mirroring the reference package layout:
  fh_gb300.sparse_for_schic      Sparse, Chrom_Dataset (contacts on the GPU)
  fh_gb300.partial_rwr           partial_rwr
  fh_gb300.project2orthogonal    project2orthogonal
  fh_gb300.parafac_integrative   parafac
  fh_gb300.parafac2_intergrative Fast_Higashi_core
All compute runs in libfhgb300.so (CUDA, sm_103a); see include/fhgb300.h for its C ABI.
"""
from ._lib import FHError, load as load_library  # noqa: F401
from .sparse_for_schic import Sparse, Chrom_Dataset  # noqa: F401
from .parafac2_intergrative import Fast_Higashi_core  # noqa: F401
from .partial_rwr import partial_rwr  # noqa: F401
from .project2orthogonal import project2orthogonal  # noqa: F401
from .parafac_integrative import parafac  # noqa: F401
