"""CPU oracle for libmarshal_gb300 -- test infrastructure, never product code."""
