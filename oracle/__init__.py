"""Test-only CPU oracle (numpy restatement of lightprop2d's propagation path).

Never imported by the ``lightprop2d_gb300`` package itself.
"""
