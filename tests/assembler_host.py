"""Test support: K-mer graphs of local-reassembly windows from the engine's
tally edges.

Mirrors Assembler.addReads / buildGraph (S/Assembler.scala:46-154) for many
windows at once: the engine tallies, for every K-mer of every recruited read
and its reverse complement, the following base with its quality and mapping
quality (pg_kmer_tally), and returns the graph edges of the K-mers with depth
>= minDepth.  The graph walk (S/Assembler.scala:164-327) stays on the host.
"""
NIB = "=ACMGRSVTWYHKDBN"


def kmer_string(hi, lo, K):
    """4-bit key words -> K-mer string."""
    out = []
    for j in range(K):
        w = hi if j < 16 else lo
        out.append(NIB[(int(w) >> (60 - 4 * (j % 16))) & 15])
    return "".join(out)


class Assembler:
    """One Assembler per window, all windows tallied in one engine call."""

    def __init__(self, engine, K=31, min_depth=5):
        self.engine = engine
        self.K = K
        self.min_depth = min_depth
        self.windows = []

    def add_reads(self, read_begin, read_end):
        """Assembler.addReads for the reads [read_begin, read_end) of the engine's
        read store; returns the window index."""
        self.windows.append((int(read_begin), int(read_end)))
        return len(self.windows) - 1

    def build_graph(self, params):
        """Assembler.buildGraph for every window: a list of (kGraph, altGraph)
        dicts K-mer -> next K-mer."""
        edges = self.engine.kmer_tally(self.windows, self.K, params, self.min_depth)
        graphs = [({}, {}) for _ in self.windows]
        for e in edges:
            k = kmer_string(e["key_hi"], e["key_lo"], self.K)
            kg, ag = graphs[int(e["window"])]
            kg[k] = k[1:] + "ACGT"[int(e["next"])]
            if int(e["alt"]) >= 0:
                ag[k] = k[1:] + "ACGT"[int(e["alt"])]
        return graphs
