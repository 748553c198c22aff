"""CPU FP64 oracle of the full-3D collocation BEM (test infrastructure only)."""
