"""CPU oracle for the MDZ hot path (test infrastructure only)."""
