"""CPU oracle of the opencl-sph per-substep pipeline.

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke()
(to check its results) and by bench.py's CPU-baseline legs; never by the
product.
oracle.py wraps the C restatement (sph_oracle.c); ref.py wraps the
reference's own code compiled by make_ref.py into oracle/_ref/.
"""
