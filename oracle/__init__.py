"""CPU oracle for the ray pipeline — TEST INFRASTRUCTURE ONLY.

A restatement of WoodenPBREngine's hot-path arithmetic used as the checker by
tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg. The product
(woodenpbrengine_gb300) never imports it. Parity status: unpinned (the
reference cannot be compiled here and ships no golden vectors)."""
