"""Sharding by owned node ranges on world_size 2 (gloo, CPU only).

The reference distributes the builder by owned node ranges: every rank builds the CSR rows of its
owned dofs from its overlap elements, with no exchange of tangent values
(``src/slope_stability/fem/distributed_tangent.py:297-478``).  Here two gloo ranks each build the
owned-row pattern of half the nodes with the host pattern builder and evaluate their rows with the
oracle (CPU); rank 0 gathers the rows and they must equal the single-rank rows bit for bit.  This
is the host-side logic of a sharded multi-GPU run (one rank per GPU, no data-path collective); it
needs no GPU.

The BDDC case (``src/slope_stability/fem/distributed_tangent.py`` ``prepare_bddc_subdomain_pattern``)
gives each rank the elements it owns and a local square matrix over their nodes; the subdomain
matrices, summed through their local-to-global dof maps, must give the whole-mesh tangent.  The
potential energy (``ConstitutiveOperator.potential_energy`` across ranks) sums each rank's owned
elements and all-reduces the scalar.
"""

from __future__ import annotations

import os
import socket

import numpy as np

from slope_stability_petsc4py_gb300 import fem, synthetic


def _problem():
    mats = synthetic.MaterialSet.homogeneous(c0=6.0, phi=35.0, young=2.0e4, poisson=0.3)
    mesh = synthetic.slope_mesh_3d(4, 2, 3, elem_type="P2")
    U = synthetic.displacement_field(mesh, mats, amplitude=0.02, seed=5)
    return mats, mesh, U


def _rows(n_range):
    """Owned-row force and tangent values of the node range, evaluated by the oracle."""
    from oracle import oracle_py as oracle
    from slope_stability_petsc4py_gb300.distributed_tangent import _PatternBuild

    mats, mesh, U = _problem()
    pb = _PatternBuild(mesh.elem, mesh.q_mask, n_range)
    g = {k: pb.get(k) for k in ("overlap_elements", "overlap_nodes", "overlap_element_dof_lids", "owned_local_overlap_dofs",
                                "indptr", "indices", "row_slot_ptr", "slot_elem", "slot_lrow", "slot_pos")}
    nnz = pb.sizes["nnz"]
    pb.close()
    xi, wf = fem.quadrature(3, "P2")
    n_q = xi.shape[1]
    dphi, w = oracle.geometry(mesh.coord, mesh.elem[:, g["overlap_elements"]], 3, fem.reference_gradients(3, "P2"), wf)
    nodes = g["overlap_nodes"]
    gdofs = 3 * np.repeat(nodes, 3) + np.tile(np.arange(3), nodes.size)
    u_ov = np.ascontiguousarray(U.reshape(-1, order="F")[gdofs])
    E = oracle.strain_3d(dphi[0], dphi[1], dphi[2], u_ov, g["overlap_element_dof_lids"], n_q)
    n = E.shape[0]
    shear = np.full(n, float(mats.shear[0]))
    lame = np.full(n, float(mats.lame[0]))
    c_bar, sin_phi = oracle.reduction(np.full(n, float(mats.c0[0])), np.full(n, np.deg2rad(float(mats.phi[0]))),
                                      np.zeros(n), 1.1, "B")
    S, DS = oracle.constitutive_3d(E, c_bar, sin_phi, shear, shear, lame)
    F = oracle.force_rows_3d(dphi[0], dphi[1], dphi[2], S, w, g["row_slot_ptr"], g["slot_elem"], g["slot_lrow"], n_q)
    K = oracle.tangent_rows_3d(dphi[0], dphi[1], dphi[2], DS, w, g["row_slot_ptr"], g["slot_elem"], g["slot_lrow"],
                               g["slot_pos"], n_q, nnz)
    rows = gdofs[g["owned_local_overlap_dofs"]]
    return rows, F, g["indptr"], g["indices"], K


def _rank_main(rank, world, port, queue):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    _, mesh, _ = _problem()
    n_nodes = mesh.n_nodes
    n0, n1 = rank * n_nodes // world, (rank + 1) * n_nodes // world
    mine = _rows((n0, n1))
    gathered = [None] * world
    dist.all_gather_object(gathered, mine)
    if rank == 0:
        queue.put(gathered)
    dist.barrier()
    dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_gloo_ranks_build_the_single_rank_rows():
    import torch.multiprocessing as mp

    from oracle import oracle_py as oracle

    oracle.build()
    ctx = mp.get_context("spawn")
    queue = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, queue)) for r in range(2)]
    for p in procs:
        p.start()
    parts = queue.get(timeout=300)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    _, mesh, _ = _problem()
    rows1, F1, ip1, ix1, K1 = _rows((0, mesh.n_nodes))
    rows = np.concatenate([p[0] for p in parts])
    assert np.array_equal(np.sort(rows), np.sort(rows1)) and rows.size == rows1.size  # a partition of the rows
    pos1 = {int(r): i for i, r in enumerate(rows1)}
    for rows_r, F_r, ip_r, ix_r, K_r in parts:
        for i, r in enumerate(rows_r):
            j = pos1[int(r)]
            assert F_r[i] == F1[j]
            a, b = ip_r[i], ip_r[i + 1]
            a1, b1 = ip1[j], ip1[j + 1]
            assert np.array_equal(ix_r[a:b], ix1[a1:b1])  # same global columns, same order
            assert np.array_equal(K_r[a:b], K1[a1:b1])


# ---------------------------------------------------------------------------- BDDC subdomains


def _bddc_local(n_range):
    """A rank's non-overlapping subdomain (host structure) and its local square tangent values,
    evaluated by the oracle: DS from the return mapping of the points' strains."""
    from oracle import oracle_py as oracle
    from slope_stability_petsc4py_gb300.bddc import bddc_local_structure

    mats, mesh, U = _problem()
    xi, wf = fem.quadrature(3, "P2")
    n_q = xi.shape[1]
    s = bddc_local_structure(mesh.coord, mesh.elem, mesh.q_mask, n_range, n_q=n_q)
    nodes, elem_local = s["local_nodes"], s["elem_local"]
    dphi, w = oracle.geometry(mesh.coord[:, nodes], elem_local, 3, fem.reference_gradients(3, "P2"), wf)
    dof = (3 * elem_local.T[:, :, None] + np.arange(3)[None, None, :]).reshape(elem_local.shape[1], -1).astype(np.int32)
    u_loc = np.ascontiguousarray(U.reshape(-1, order="F")[s["local_global_dofs"]])
    E = oracle.strain_3d(dphi[0], dphi[1], dphi[2], u_loc, dof, n_q)
    n = E.shape[0]
    shear, lame = np.full(n, float(mats.shear[0])), np.full(n, float(mats.lame[0]))
    c_bar, sin_phi = oracle.reduction(np.full(n, float(mats.c0[0])), np.full(n, np.deg2rad(float(mats.phi[0]))),
                                      np.zeros(n), 1.1, "B")
    _, DS = oracle.constitutive_3d(E, c_bar, sin_phi, shear, shear, lame)
    lp = s["local_matrix_pattern"]
    K = oracle.tangent_scatter(3, dphi[0], dphi[1], dphi[2], DS, w, s["scatter_map"], n_q, lp.nnz)
    K[s["constrained_diag_positions"]] = 1.0
    return {"elements": s["local_elements"], "gdofs": s["local_global_dofs"], "free": s["free_local"],
            "indptr": lp.indptr, "indices": lp.indices, "values": K}


def _bddc_rank_main(rank, world, port, queue, split):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    _, mesh, _ = _problem()
    bounds = [0, split, mesh.n_nodes]
    mine = _bddc_local((bounds[rank], bounds[rank + 1]))
    gathered = [None] * world
    dist.all_gather_object(gathered, mine)
    if rank == 0:
        queue.put(gathered)
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_bddc_subdomains_sum_to_the_global_tangent():
    """Each rank owns the elements whose smallest node lies in its node range: the subdomains
    partition the elements, and their local square tangents, summed through the local-to-global
    dof maps, give the single-subdomain (whole-mesh) tangent on the free dofs."""
    import torch.multiprocessing as mp
    from scipy.sparse import coo_matrix, csr_matrix

    from oracle import oracle_py as oracle

    oracle.build()
    _, mesh, _ = _problem()
    owners = np.sort(mesh.elem.min(axis=0))
    split = int(owners[owners.size // 2])
    ctx = mp.get_context("spawn")
    queue = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_bddc_rank_main, args=(r, 2, port, queue, split)) for r in range(2)]
    for p in procs:
        p.start()
    parts = queue.get(timeout=300)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    elems = np.concatenate([p["elements"] for p in parts])
    assert np.array_equal(np.sort(elems), np.arange(mesh.n_elem))  # a partition of the elements
    assert all(p["elements"].size > 0 for p in parts)
    n_dof = 3 * mesh.n_nodes
    free = mesh.q_mask.reshape(-1, order="F")

    def assemble(p):
        A = csr_matrix((p["values"], p["indices"], p["indptr"]), shape=(p["gdofs"].size,) * 2).tocoo()
        keep = p["free"][A.row] & p["free"][A.col]  # the free-free block (Dirichlet rows are local identities)
        return coo_matrix((A.data[keep], (p["gdofs"][A.row[keep]], p["gdofs"][A.col[keep]])), shape=(n_dof, n_dof))

    K_sum = (assemble(parts[0]) + assemble(parts[1])).tocsr()
    K_one = assemble(_bddc_local((0, mesh.n_nodes))).tocsr()
    diff = abs(K_sum - K_one).max()
    assert diff <= 1e-12 * abs(K_one).max()
    assert K_one[free][:, free].nnz > 0 and K_sum[~free].nnz == 0


# ---------------------------------------------------------------------------- potential energy


def _potential_part(n_range):
    """The rank's share of the integrated potential energy: the oracle's energy densities at the
    points of the overlap elements the range owns (owned_element_mask), weighted and summed."""
    from oracle import oracle_py as oracle
    from slope_stability_petsc4py_gb300.distributed_tangent import _PatternBuild, owned_element_mask

    mats, mesh, U = _problem()
    pb = _PatternBuild(mesh.elem, mesh.q_mask, n_range)
    g = {k: pb.get(k) for k in ("overlap_elements", "overlap_nodes", "overlap_element_dof_lids")}
    pb.close()
    xi, wf = fem.quadrature(3, "P2")
    n_q = xi.shape[1]
    dphi, w = oracle.geometry(mesh.coord, mesh.elem[:, g["overlap_elements"]], 3, fem.reference_gradients(3, "P2"), wf)
    nodes = g["overlap_nodes"]
    gdofs = 3 * np.repeat(nodes, 3) + np.tile(np.arange(3), nodes.size)
    u_ov = np.ascontiguousarray(U.reshape(-1, order="F")[gdofs])
    E = oracle.strain_3d(dphi[0], dphi[1], dphi[2], u_ov, g["overlap_element_dof_lids"], n_q)
    n = E.shape[0]
    c_bar, sin_phi = oracle.reduction(np.full(n, float(mats.c0[0])), np.full(n, np.deg2rad(float(mats.phi[0]))),
                                      np.zeros(n), 1.1, "B")
    full = lambda v: np.full(n, float(v[0]))  # noqa: E731
    psi = oracle.potential_3d(E.T, c_bar, sin_phi, full(mats.shear), full(mats.bulk), full(mats.lame))
    own = np.repeat(owned_element_mask(mesh.elem, g["overlap_elements"], n_range), n_q)
    return float(np.dot(w[own], psi[own])), g["overlap_elements"][owned_element_mask(mesh.elem, g["overlap_elements"],
                                                                                       n_range)]


def _potential_rank_main(rank, world, port, queue, split):
    import torch
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    _, mesh, _ = _problem()
    bounds = [0, split, mesh.n_nodes]
    part, owned = _potential_part((bounds[rank], bounds[rank + 1]))
    buf = torch.tensor([part], dtype=torch.float64)
    dist.all_reduce(buf)  # the exchange the operator's potential_energy does across ranks
    gathered = [None] * world
    dist.all_gather_object(gathered, owned)
    if rank == 0:
        queue.put((float(buf.item()), gathered))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_potential_energy_sums_to_the_whole_mesh():
    """Two ranks splitting the node range at the median element owner (vertices are numbered
    before edge nodes, so half the node range would own no element): the elements they own
    partition the mesh, and their all-reduced energies equal the single-rank energy of the whole
    mesh."""
    import torch.multiprocessing as mp

    from oracle import oracle_py as oracle

    oracle.build()
    _, mesh, _ = _problem()
    split = int(np.sort(mesh.elem.min(axis=0))[mesh.n_elem // 2])
    ctx = mp.get_context("spawn")
    queue = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_potential_rank_main, args=(r, 2, port, queue, split)) for r in range(2)]
    for p in procs:
        p.start()
    total, owned = queue.get(timeout=300)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    elems = np.concatenate(owned)
    assert np.array_equal(np.sort(elems), np.arange(mesh.n_elem)) and all(o.size for o in owned)
    whole, _ = _potential_part((0, mesh.n_nodes))
    assert abs(total - whole) <= 1e-12 * abs(whole)
