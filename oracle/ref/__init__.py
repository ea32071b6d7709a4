"""Build recipe, harness and file formats for running the reference's own
CUDARenderer as an oracle (test infrastructure only)."""
