"""Oracle package: the FP64 CPU restatement of rust_qmc's walker path.

TEST INFRASTRUCTURE.  Only tests/, __graft_entry__.smoke() and the bench's
CPU-baseline leg may import this package; the product never does.
"""
