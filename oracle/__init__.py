"""CPU oracle for the parity tests (test infrastructure only; never imported by the
engine).  See oracle/pe_oracle.h."""
