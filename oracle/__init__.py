"""CPU oracle of the Rot2D3C hot path: TEST INFRASTRUCTURE ONLY (see rot2d3c_oracle)."""
