"""CPU oracle of the MLS-MPM substep (test infrastructure only)."""
