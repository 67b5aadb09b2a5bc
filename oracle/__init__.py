"""CPU oracle for the SIMP path (test infrastructure only)."""
