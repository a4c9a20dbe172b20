"""Timing tables and trained weights of the learned schedule tuner, and the scripts that made
them (build_dataset.py on a GB300, then train.py)."""
