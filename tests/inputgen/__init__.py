"""TEST AND BENCH INFRASTRUCTURE: inputs for the tests and the benchmark (not
part of the product)."""
