"""CPU oracle for the fused D3Q19 step (test infrastructure only; never part of the product path)."""
