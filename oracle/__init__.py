"""ORACLE -- test infrastructure, never part of the product.

oracle/port: C restatement of the reference hot path (built by
oracle/Makefile into oracle/_build/libmahyco_port.so); oracle/port.py binds it.
oracle/ref_harness.cc + oracle/Makefile.ref: the reference itself, compiled
from its own sources against oracle/kokkos_shim, used here to generate and
check golden vectors (it cannot run on hosts without the reference sources).
"""
