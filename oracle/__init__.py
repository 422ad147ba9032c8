"""CPU oracle for the implicit MPM snow substep (test infrastructure only)."""
