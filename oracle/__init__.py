"""TEST INFRASTRUCTURE: the CPU oracle (checker) -- never imported by the product."""
