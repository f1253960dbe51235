"""CPU oracle of the mpx SRBD-MPC hot path (test infrastructure only)."""
