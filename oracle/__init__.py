"""BQSR oracle — test infrastructure only (CPU restatement of the reference; see bqsr_oracle.h)."""
