"""CPU oracle for the DRR + similarity-metric path (test infrastructure only)."""
