"""CPU oracle of the path-tracing core. TEST INFRASTRUCTURE: imported by tests, the smoke
check and the benchmark's CPU-baseline leg only; never by the product package."""
