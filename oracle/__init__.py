"""CPU oracle -- test infrastructure only.

A sequential restatement of the reference's progressive UMAP path
(``gm_oracle.cpp``, loaded by ``oracle.session``), the FP64 brute-force k-NN
and quality metrics (``oracle.knn``).  Only tests, the smoke check and the
benchmark's CPU-baseline leg use it.
"""
