"""The oracle: a CPU restatement of the reference's RSVD path, used only by
tests/, the smoke check and the benchmark's CPU-baseline leg as a checker."""
