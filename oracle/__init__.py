"""CPU oracle of the voxelDVC Gauss-Newton path (test infrastructure only)."""
