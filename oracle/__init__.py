"""CPU oracle of the open-earth-benchmarks stencils (TEST INFRASTRUCTURE; see oracle.py)."""
