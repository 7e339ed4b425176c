"""CPU checkers for the isosurface path (test infrastructure, never shipped).

`oracle.lib` wraps the C restatement in c3d_oracle.c; `oracle.ref` wraps the
reference library compiled from its own sources (available only where the
reference tree was present at build time).
"""
