"""CPU oracle for libtrixi_b200.so -- test infrastructure only (see trixi_oracle.c)."""
