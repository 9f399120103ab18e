"""CPU oracle for the DPM time step (test infrastructure only)."""
