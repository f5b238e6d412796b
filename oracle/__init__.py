"""CPU oracle for the probebwa mapping path (test infrastructure only)."""
