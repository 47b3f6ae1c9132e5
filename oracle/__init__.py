"""CPU oracle for the block-sparse hot path (test infrastructure only)."""
