"""CPU oracle for the lvr2 reconstruction hot path (test infrastructure only)."""
