"""CPU oracle for the parquet-iteration hot path (test infrastructure only; never shipped)."""
