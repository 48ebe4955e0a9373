"""CPU oracle for the RDC-XPBD substep (test infrastructure only; never imported by the product)."""
