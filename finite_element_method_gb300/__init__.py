"""GB300-native (sm_103a, FP64) element-stiffness-and-assembly path of the
Rust crate `finite_element_method`, behind a C ABI (include/fem_gpu.h).

`FEM` mirrors the crate's FEM::create / add_node / add_truss / add_beam /
add_plate API; `meshes` generates the seeded synthetic workloads.
"""
from .fem import FEM, Batch, FEMError, SeparatedStiffnessSparse  # noqa: F401

__all__ = ["FEM", "Batch", "FEMError", "SeparatedStiffnessSparse"]
