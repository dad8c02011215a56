"""CPU oracle: restatement of the reference algorithm (restate.c) and the recipe
that builds the reference runtime itself (ref.mk).  Test infrastructure only."""
