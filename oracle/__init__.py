"""ORACLE — test infrastructure (CPU restatement of the reference, golden
loaders, reference MEX tracer host).  The engine package never imports it."""
