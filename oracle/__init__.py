"""FP64 CPU oracle of the reference's solve path (test infrastructure only)."""
