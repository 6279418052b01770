"""CPU oracle for the DAMASK_grid spectral path (test infrastructure only)."""
