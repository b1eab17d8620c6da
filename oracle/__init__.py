"""Test infrastructure: the CPU oracle, the reference harness and the
reference GPU kernel runner.  Never imported by the product package."""
