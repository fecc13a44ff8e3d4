"""The reference's own kernel code on the CPU (test infrastructure; see build_refexec.py)."""
