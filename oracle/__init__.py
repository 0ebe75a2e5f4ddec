"""CPU oracle for the ForkMatch hot path: test infrastructure only."""
