"""ORACLE package -- test infrastructure only: the CPU restatement of SeeSharp's PathTracer path
used to check the CUDA implementation.  Only tests/, the smoke check and bench.py's CPU-baseline
leg import it."""
