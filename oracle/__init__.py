"""CPU oracle for tack-lbm's D3Q19 step: test infrastructure, never the product."""
