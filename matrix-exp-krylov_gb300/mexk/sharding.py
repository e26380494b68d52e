"""Row sharding of the restarted-Arnoldi solve over several ranks: the
partition, the halo (ghost) plan and the two exchanges a sharded Arnoldi step
needs.

The reference splits A into 1D row blocks (CSRHost::partition_rows,
main.cu:526-562), gives each GPU the list of x entries it must receive from
every other one and send to it (build_owner_ghost_maps, main.cu:587-691,
checked pairwise by validate_ghost_maps, main.cu:695-744), exchanges q_j over
peer copies before every SpMV (ghost_exchange_qj, main.cu:1635-1720) and
reduces every dot product of its Gram-Schmidt passes with its own scalar
NCCL allreduce (main.cu:1193-1218, 1596, 1808, 1846, 1892): 2(j+1)+1
collectives per step.

Here a rank holds its row block with the columns renumbered into one local
index space -- owned columns first, then the ghosts in owner order -- so the
local SpMV is an ordinary square-times-extended-vector product over
[x_owned | x_ghost], and a step needs one halo exchange (point-to-point, to
and from the peers the plan names) and one all-reduce per Gram-Schmidt pass
of the whole vector of that pass's dot products (plus the norm): 3 vector
collectives per step instead of 2(j+1)+1 scalar ones.

The exchanges go through torch.distributed (gloo on CPU, NCCL on GPUs). The
plan and the exchange protocol are tested with world-size-2 and -3 gloo runs
that reproduce the single-partition solve; no run of this pool has more
than one GPU, so the sharded solve on GPUs is unmeasured.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np


def partition_rows(n: int, parts: int):
    """Row ranges [start, end) of the 1D blocks: n // parts rows each, the
    remainder to the first blocks (CSRHost::partition_rows, main.cu:526-562)."""
    if parts < 1:
        raise ValueError("parts must be >= 1")
    base, extra = divmod(n, parts)
    out, start = [], 0
    for p in range(parts):
        rows = base + (1 if p < extra else 0)
        out.append((start, start + rows))
        start += rows
    return out


def owner_of(cols: np.ndarray, ranges) -> np.ndarray:
    """Rank owning each global column index."""
    starts = np.array([r[0] for r in ranges], dtype=np.int64)
    ends = np.array([r[1] for r in ranges], dtype=np.int64)
    own = np.searchsorted(ends, cols, side="right")
    if np.any(own >= len(ranges)) or np.any(cols < starts[np.minimum(own, len(ranges) - 1)]):
        raise ValueError("column index outside every row block")
    return own


@dataclass
class HaloPlan:
    """One rank's view of the sharded matrix (build_owner_ghost_maps).

    recv[o]: sorted global columns this rank needs from owner o (the
    reference's owner_to_consumer_map); send[c]: sorted global columns of its
    own block that consumer c needs (consumer_to_owner_map). The ghosts sit
    after the owned entries of the extended vector in owner order, each
    owner's in ascending column order (incoming_global_col_indices).
    row_ptr / col_idx / values: the row block with columns renumbered into
    that extended index space."""

    rank: int
    parts: int
    row_start: int
    row_end: int
    recv: dict = field(default_factory=dict)
    send: dict = field(default_factory=dict)
    recv_offsets: list = field(default_factory=list)
    send_offsets: list = field(default_factory=list)
    row_ptr: np.ndarray = None
    col_idx: np.ndarray = None
    values: np.ndarray = None

    @property
    def n_local(self) -> int:
        return self.row_end - self.row_start

    @property
    def n_ghost(self) -> int:
        return sum(len(v) for v in self.recv.values())

    def incoming(self) -> np.ndarray:
        """Flattened ghost columns in the extended vector's order."""
        parts = [self.recv[o] for o in sorted(self.recv)]
        return np.concatenate(parts) if parts else np.zeros(0, dtype=np.int64)


def build_halo_plan(row_ptr, col_idx, values, rank: int, parts: int) -> HaloPlan:
    """The halo plan of `rank` for the global CSR matrix (square, n rows)."""
    row_ptr = np.asarray(row_ptr, dtype=np.int64)
    col_idx = np.asarray(col_idx, dtype=np.int64)
    n = len(row_ptr) - 1
    ranges = partition_rows(n, parts)
    r0, r1 = ranges[rank]
    plan = HaloPlan(rank=rank, parts=parts, row_start=r0, row_end=r1)
    # receive lists: the off-block columns of my rows, per owner, unique and sorted
    my_cols = col_idx[row_ptr[r0]:row_ptr[r1]]
    off = my_cols[(my_cols < r0) | (my_cols >= r1)]
    if off.size:
        own = owner_of(off, ranges)
        for o in range(parts):
            lst = np.unique(off[own == o])
            if lst.size:
                plan.recv[o] = lst
    # send lists: the columns of my block that each other block's rows use
    for c in range(parts):
        if c == rank:
            continue
        c0, c1 = ranges[c]
        theirs = col_idx[row_ptr[c0]:row_ptr[c1]]
        need = np.unique(theirs[(theirs >= r0) & (theirs < r1)])
        if need.size:
            plan.send[c] = need
    off_r = 0
    for o in range(parts):
        plan.recv_offsets.append(off_r)
        off_r += len(plan.recv.get(o, ()))
    off_s = 0
    for c in range(parts):
        plan.send_offsets.append(off_s)
        off_s += len(plan.send.get(c, ()))
    # local CSR over [owned | ghosts]
    rp = row_ptr[r0:r1 + 1] - row_ptr[r0]
    cols = my_cols.copy()
    local = (cols >= r0) & (cols < r1)
    cols[local] -= r0
    if (~local).any():
        # owners' blocks are in rank order, so the flattened ghost list is sorted
        cols[~local] = (r1 - r0) + np.searchsorted(plan.incoming(), my_cols[~local])
    plan.row_ptr = rp.astype(np.int32)
    plan.col_idx = cols.astype(np.int32)
    plan.values = np.asarray(values, dtype=np.float64)[row_ptr[r0]:row_ptr[r1]].copy()
    return plan


def validate_plans(plans) -> None:
    """Every pair agrees: what owner o sends to consumer c is exactly what c
    expects from o (validate_ghost_maps, main.cu:695-744). Raises ValueError
    naming the first mismatching pair."""
    P = len(plans)
    for o in range(P):
        for c in range(P):
            if o == c:
                continue
            send = plans[o].send.get(c, np.zeros(0, dtype=np.int64))
            recv = plans[c].recv.get(o, np.zeros(0, dtype=np.int64))
            if not np.array_equal(np.unique(send), np.unique(recv)):
                raise ValueError(f"Ghost map mismatch between owner {o} and consumer {c}: "
                                 f"send size {len(send)}, recv size {len(recv)}")


def halo_exchange(plan: HaloPlan, x_local, group=None):
    """[x_owned | x_ghost] for this rank: sends every consumer the entries of
    x_local it needs and receives this rank's ghosts from their owners, all
    point-to-point and in flight together (the reference's q_j ghost
    exchange). x_local: a torch tensor of the rank's n_local entries."""
    import torch
    import torch.distributed as dist

    ghost = torch.empty(plan.n_ghost, dtype=x_local.dtype, device=x_local.device)
    reqs, sent = [], []  # the send buffers stay referenced until their requests complete
    for c in sorted(plan.send):
        idx = torch.as_tensor(plan.send[c] - plan.row_start, device=x_local.device)
        sent.append(x_local.index_select(0, idx).contiguous())
        reqs.append(dist.isend(sent[-1], dst=c, group=group))
    bufs = {}
    for o in sorted(plan.recv):
        bufs[o] = torch.empty(len(plan.recv[o]), dtype=x_local.dtype, device=x_local.device)
        reqs.append(dist.irecv(bufs[o], src=o, group=group))
    for r in reqs:
        r.wait()
    for o, b in bufs.items():
        a = plan.recv_offsets[o]
        ghost[a:a + b.numel()] = b
    return torch.cat([x_local, ghost])


def allreduce_sum(vec, group=None):
    """Sum of one vector over the ranks in place (one collective for all the
    dot products of a Gram-Schmidt pass)."""
    import torch.distributed as dist

    dist.all_reduce(vec, op=dist.ReduceOp.SUM, group=group)
    return vec


__all__ = ["partition_rows", "owner_of", "HaloPlan", "build_halo_plan", "validate_plans", "halo_exchange",
           "allreduce_sum"]
