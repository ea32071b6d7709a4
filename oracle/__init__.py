"""CPU oracle for the frame hot path (test infrastructure only)."""
