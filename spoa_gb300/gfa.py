"""GFA 1.0 text of a POA graph, in the layout of spoa's CLI writer.

Restates ``PrintGfa`` (src/main.cpp:119-199): one S line per node in id order
(1-based, ``ic:Z:true`` on consensus nodes) followed by that node's L lines
in out-edge order with ``ew:f:<weight>`` (``ic:Z:true`` when both ends are
consensus nodes); one P line per sequence following its labelled path
(reversed with ``-`` orientation for reads kept on the reverse strand);
optionally a ``Consensus`` P line.
"""
from __future__ import annotations


def gfa_lines(chars, edge_tail, edge_head, edge_weight, paths, consensus,
              is_reversed=None, headers=None, include_consensus=True):
    """chars[i]: decoded node character (int or bytes); edge_* in node-major
    out-edge order; paths[s]: node ids of sequence s; consensus: node ids."""
    n = len(chars)
    is_cons = [False] * n
    for v in consensus:
        is_cons[int(v)] = True
    out = ["H\tVN:Z:1.0"]
    e = 0
    ne = len(edge_tail)
    for i in range(n):
        line = f"S\t{i + 1}\t{chr(int(chars[i]))}"
        if is_cons[i]:
            line += "\tic:Z:true"
        out.append(line)
        while e < ne and int(edge_tail[e]) == i:
            h = int(edge_head[e])
            line = f"L\t{i + 1}\t+\t{h + 1}\t+\tOM\tew:f:{int(edge_weight[e])}"
            if is_cons[i] and is_cons[h]:
                line += "\tic:Z:true"
            out.append(line)
            e += 1
    for s, path in enumerate(paths):
        name = headers[s] if headers is not None else f"read{s}"
        ids = [int(v) + 1 for v in path]
        ir = bool(is_reversed[s]) if is_reversed is not None and len(is_reversed) else False
        if ir:
            ids.reverse()
        body = ",".join(f"{v}{'-' if ir else '+'}" for v in ids)
        out.append(f"P\t{name}\t{body}\t*")
    if include_consensus:
        body = ",".join(f"{int(v) + 1}+" for v in consensus)
        out.append(f"P\tConsensus\t{body}\t*")
    return out
