"""Test infrastructure: CPU restatements of the reference used only to check the engine."""
