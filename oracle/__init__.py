"""FP64 CPU oracle of the Bartels tet-mesh path (test infrastructure only)."""
