"""Known-answer accuracy harness (ground_truth/ of the reference): make a
deformed image from a reference and a known displacement, run the usual
preprocess -> run pipeline on it, and score the recovered displacement."""
