"""GB300-native BEM Galerkin matrix assembly (drop-in for BEASTGPU's assemble_gpu path)."""
from .meshes import Mesh, icosphere, ellipsoid, plate, two_plates, ellipsoid_batch  # noqa: F401
from .spaces import Space, raviartthomas, lagrangec0d1, REFSPACE_RT, REFSPACE_LAGRANGE_C0D1  # noqa: F401
from .operators import Helmholtz3D, Maxwell3D, Operator, QuadStrat, defaultquadstrat  # noqa: F401
from .api import (assemble_gpu, assemble, classify, local_matrices, GPUConfiguration, row_shard,  # noqa: F401
                  GpuWriteBackTrueInstance, GpuWriteBackFalseInstance, measure_issue_peaks, Batch,
                  assemble_batch)
