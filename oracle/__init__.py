"""FP64 CPU oracle for FeeLLGood's per-time-step LLG path. TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may import this
package. The product (feellgood_gb300) never imports, links or calls it.
"""
