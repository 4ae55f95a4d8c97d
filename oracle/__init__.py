"""The CPU oracle of the GRIS path (test infrastructure only).

gris_oracle.cpp   C++ restatement of the reference's GLSL hot path (built by build_oracle.py)
detmath.h         deterministic sin/cos/tan shared by the oracle's restatement and harness
ref/              recipe that compiles the reference's own shaders as C++ (pinning reference)
pyoracle.py       Python driver of both (renderer frame loop, ray queries)

Only tests/, __graft_entry__.smoke() and bench.py's CPU legs may import this package.
"""
