"""Domain decomposition of the lattice in t with halo exchange (host side).

How the path shards across GPUs (MILC's layout_hyper_prime.c splits the
lattice into one sub-lattice per rank; dslash_fn_field gathers the
neighbour faces, com_mpi.c): rank r of R holds t in [r*T, (r+1)*T), T =
nt/R, as a local lattice extended by H = 4 ghost slices on each side
(depth 3 for the Naik term, even so that the local checkerboard parity of
a site equals its global parity).  A D_eo application on rank r is the
single-GPU kernel run on the extended local lattice after the ghost slices
of the input vector (and, once per link load, of the links) were filled
from the neighbouring ranks; the results on the interior sites equal those
of the global operator exactly, because every site's arithmetic is the
same.  A CG over the decomposition adds one global sum per dot product.

This module holds the index maps and the pack / exchange / unpack steps on
host (numpy) fields; the exchange itself goes through torch.distributed
point-to-point calls, or a direct copy when both sub-domains live in one
process.  Faces are packed and unpacked on the host; with the NCCL backend
(one GPU per rank) they travel as device tensors, with gloo as host tensors.
"""
import numpy as np

GHOST = 4


def _site_index_table(dims):
    """MILC index of every site, as a lexicographic (t, z, y, x) array:
    lexicographic i = x + nx (y + ny (z + nz t)); even sites (x+y+z+t even)
    at i/2, odd sites at (i + V)/2 (generic/layout_hyper_prime.c:509-520,
    the same map as mks_site_index)."""
    nx, ny, nz, nt = dims
    V = nx * ny * nz * nt
    t, z, y, x = np.meshgrid(np.arange(nt), np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    i = x + nx * (y + ny * (z + nz * t))
    odd = ((x + y + z + t) & 1).astype(bool)
    return np.where(odd, (i + V) // 2, i // 2).astype(np.int64)


class TSlabs:
    """R sub-domains along t of a (nx, ny, nz, nt) lattice."""

    def __init__(self, dims, nranks, ghost=GHOST):
        nx, ny, nz, nt = dims
        if nt % nranks or (nt // nranks) % 2 or ghost % 2 or ghost < 3:
            raise ValueError("nt must split into even slabs, ghost depth even and >= 3")
        self.dims, self.R, self.H = tuple(dims), nranks, ghost
        self.T = nt // nranks
        if self.T < ghost:
            raise ValueError("slab thinner than the ghost zone")
        self.local_dims = (nx, ny, nz, self.T + 2 * ghost)
        self.gidx = _site_index_table(self.dims)          # global MILC index by (t, z, y, x)
        self.lidx = _site_index_table(self.local_dims)    # local MILC index by (t_ext, z, y, x)

    def global_t(self, rank, t_ext):
        return (rank * self.T + t_ext - self.H) % self.dims[3]

    def interior(self):
        """Local MILC indices of the interior slices, (t, z, y, x)-ordered."""
        return self.lidx[self.H:self.H + self.T].reshape(-1)

    def interior_global(self, rank):
        return self.gidx[rank * self.T:(rank + 1) * self.T].reshape(-1)

    def scatter(self, field, rank):
        """Local extended field (ghosts filled from the global field)."""
        Vl = int(np.prod(self.local_dims))
        out = np.zeros((Vl,) + field.shape[1:], dtype=field.dtype)
        for te in range(self.local_dims[3]):
            out[self.lidx[te].reshape(-1)] = field[self.gidx[self.global_t(rank, te)].reshape(-1)]
        return out

    def scatter_interior(self, field, rank):
        """Local extended field with only the interior filled (ghosts zero)."""
        Vl = int(np.prod(self.local_dims))
        out = np.zeros((Vl,) + field.shape[1:], dtype=field.dtype)
        out[self.interior()] = field[self.interior_global(rank)]
        return out

    def gather_interior(self, local, rank, out):
        out[self.interior_global(rank)] = local[self.interior()]
        return out

    # ---- faces ----
    def face_send(self, local, side):
        """The H slices a neighbour needs: side -1 -> the lower interior
        slices (for the rank below), +1 -> the upper interior slices."""
        H, T = self.H, self.T
        sl = range(H, 2 * H) if side < 0 else range(T, T + H)
        return np.stack([local[self.lidx[t].reshape(-1)] for t in sl])

    def face_recv(self, local, side, face):
        """Store a neighbour's face into the ghost slices below (side -1) or
        above (side +1)."""
        H, T = self.H, self.T
        sl = range(0, H) if side < 0 else range(T + H, T + 2 * H)
        for k, t in enumerate(sl):
            local[self.lidx[t].reshape(-1)] = face[k]
        return local

    def exchange_local(self, locals_):
        """Halo exchange when every sub-domain lives in this process."""
        R = self.R
        up = [self.face_send(locals_[r], +1) for r in range(R)]
        down = [self.face_send(locals_[r], -1) for r in range(R)]
        for r in range(R):
            self.face_recv(locals_[r], -1, up[(r - 1) % R])
            self.face_recv(locals_[r], +1, down[(r + 1) % R])
        return locals_

    def exchange_dist(self, local, rank):
        """Halo exchange with torch.distributed (one rank per sub-domain).
        The faces travel as tensors on the backend's device: CUDA tensors for
        NCCL (which carries device memory only), host tensors for gloo."""
        import torch
        import torch.distributed as dist
        R = self.R
        dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
        up, down = self.face_send(local, +1), self.face_send(local, -1)
        t_up = torch.from_numpy(np.ascontiguousarray(up)).to(dev)
        t_down = torch.from_numpy(np.ascontiguousarray(down)).to(dev)
        t_lo, t_hi = torch.empty_like(t_up), torch.empty_like(t_down)
        ops = [dist.P2POp(dist.isend, t_up, (rank + 1) % R), dist.P2POp(dist.irecv, t_lo, (rank - 1) % R),
               dist.P2POp(dist.isend, t_down, (rank - 1) % R), dist.P2POp(dist.irecv, t_hi, (rank + 1) % R)]
        for req in dist.batch_isend_irecv(ops):
            req.wait()
        self.face_recv(local, -1, t_lo.cpu().numpy())
        self.face_recv(local, +1, t_hi.cpu().numpy())
        return local
