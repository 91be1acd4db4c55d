"""TEST INFRASTRUCTURE ONLY: the CPU oracle (see pdl_oracle.c)."""
