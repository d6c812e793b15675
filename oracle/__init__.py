"""Test infrastructure: CPU restatement of the reference hot path (the oracle)."""
