"""TEST INFRASTRUCTURE: the CPU oracle (C restatement of the reference path).  Not product code."""
