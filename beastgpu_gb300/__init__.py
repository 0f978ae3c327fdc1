"""GB300-native BEM Galerkin matrix assembly (drop-in for BEASTGPU's assemble_gpu path)."""
from .meshes import Mesh, icosphere, ellipsoid, plate, two_plates, ellipsoid_batch, meshcuboid  # noqa: F401
from .spaces import Space, raviartthomas, lagrangec0d1, lagrangecxd0, REFSPACE_RT, REFSPACE_LAGRANGE_C0D1  # noqa: F401
from .operators import Helmholtz3D, Maxwell3D, Operator, QuadStrat, defaultquadstrat  # noqa: F401
from .api import (assemble_gpu, assemble, classify, local_matrices, GPUConfiguration, row_shard,  # noqa: F401
                  GpuWriteBackTrueInstance, GpuWriteBackFalseInstance, measure_issue_peaks, Batch,
                  assemble_batch, local_matrices_curve)
from .curves import (CurveMesh, CurveSpace, circle, ellipse, arc, union, curve_lagrangec0d1,  # noqa: F401
                     curve_lagrangecxd0, Helmholtz2D, Operator2D, QuadStrat2D, defaultquadstrat2d)
