"""UNSFlow2D residual-and-update hot path on GB300 (sm_103a).

    unsflow2d_gb300.solver   CCSolver / NCSolver: the drop-in entry points
    unsflow2d_gb300.mesh     airfoil O-meshes, geometry.inp, geometric
    unsflow2d_gb300.abi      ctypes mirror of include/*.h
    unsflow2d_gb300.build    in-tree build of the two shared libraries
"""
__all__ = ["abi", "mesh", "solver", "build"]
