"""CPU oracles for the iVR hot path (test infrastructure only)."""
