"""CPU oracle (test infrastructure only): a NumPy/LAPACK restatement of Qrochet.jl's Chain path."""
