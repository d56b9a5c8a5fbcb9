"""Test infrastructure: the CPU oracle (see oracle/oracle.h)."""
