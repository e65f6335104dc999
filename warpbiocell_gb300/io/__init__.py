"""Run directories, metrics files and checkpoints."""
