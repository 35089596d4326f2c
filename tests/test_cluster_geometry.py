"""The index arithmetic of the thread-block cluster form (csrc/mcx_cluster.cu), restated on
the CPU: for every cluster size the host may choose, each CTA's shared-memory accesses
(own units, halo units, the neighbours' halos written through distributed shared memory)
stay inside its slab and are aligned for the chunk width, every local row a chunk reads is
the global neighbour row the checkerboard rule names (ising.jl:119-121 neighbour lists of
Graphs.grid(dims; periodic=true)), and every unit is owned by exactly one CTA."""
import pytest

K_SMALL = 16384  # most sites of a colour one CTA holds


def small_width(W, sites):
    for V in (16, 8):
        if W % V == 0 and sites // V >= 256:
            return V
    return 4


def cluster_sizes(dims):
    """(C, V, threads, slab) for every cluster size the host loop may take."""
    dim = len(dims)
    Lx, Ly = dims[0], dims[1]
    Lz = dims[2] if dim == 3 else 1
    W = Lx // 2
    units = Ly if dim == 2 else Lz
    U = 1 if dim == 2 else Ly
    unitB = U * W
    out = []
    for C in range(min(16, units), 1, -1):
        per = -(-units // C) * unitB
        if per > K_SMALL:
            break
        V = small_width(W, per)
        T = min(512, max(32, (per // V + 31) & ~31))
        slab = ((-(-units // C) + 2) * unitB + 15) & ~15
        assert 2 * ((per + 2 * unitB + 15) & ~15) == 2 * slab  # host smem == device slabs
        out.append((C, V, T, slab))
    return out


def check_geometry(dims, C, V, T, slab):
    dim = len(dims)
    Lx, Ly = dims[0], dims[1]
    Lz = dims[2] if dim == 3 else 1
    W = Lx // 2
    half = Ly * Lz * W
    units = Ly if dim == 2 else Lz
    U = 1 if dim == 2 else Ly
    unitB = U * W
    cpr = W // V
    fu = lambda b: units * b // C
    owned = []
    for k in range(C):
        u0, nu = fu(k), fu(k + 1) - fu(k)
        assert nu >= 1
        owned.extend(range(u0, u0 + nu))
        kp, kn = (k - 1) % C, (k + 1) % C
        nu_p = fu(kp + 1) - fu(kp)
        # kp's bottom halo (its local unit nu_p + 1) is this CTA's first unit; kn's top
        # halo (its local unit 0) is this CTA's last unit
        assert (fu(kp) + nu_p) % units == u0
        assert (fu(kn) - 1) % units == (u0 + nu - 1) % units
        assert (nu + 2) * unitB <= slab and slab % 16 == 0

        def l2g(X):  # local row -> global row
            lu, yx = divmod(X, U)
            gu = (u0 - 1 + lu) % units
            return gu if dim == 2 else yx + U * gu

        for g in range(nu * U * cpr):
            q, r0 = g % cpr, g // cpr
            y, z = r0 % U, r0 // U
            lu = z + 1
            for c in (0, 1):
                if dim == 2:
                    gy = u0 + z
                    lr, gr, p = lu, gy, (gy + c) & 1
                    pairs = [(lr + 1, (gy + 1) % Ly), (lr - 1, (gy - 1) % Ly)]
                else:
                    gz = u0 + z
                    lr, gr, p = y + U * lu, y + U * gz, (y + gz + c) & 1
                    pairs = [((y + 1) % U + U * lu, (y + 1) % Ly + Ly * gz),
                             ((y - 1) % U + U * lu, (y - 1) % Ly + Ly * gz),
                             (y + U * (lu + 1), y + Ly * ((gz + 1) % Lz)),
                             (y + U * (lu - 1), y + Ly * ((gz - 1) % Lz))]
                assert l2g(lr) == gr
                for X, G in pairs:
                    assert 0 <= X * W and X * W + W <= slab
                    assert l2g(X) == G
                k0 = q * V
                assert (lr * W + k0) % min(V, 16) == 0 and lr * W + k0 + V <= slab
                ke = (W - 1 if k0 == 0 else k0 - 1) if p == 0 else (0 if k0 + V == W else k0 + V)
                assert 0 <= lr * W + ke < slab
                assert gr * W + k0 + V <= half
                uoff = y * W + k0
                if z == 0:
                    o = (nu_p + 1) * unitB + uoff
                    assert o % min(V, 16) == 0 and o + V <= slab
                if z == nu - 1:
                    assert uoff + V <= unitB
    assert sorted(owned) == list(range(units))
    # per-warp sums of the per-sweep deltas fit in int32 (at most 12 per site and sweep)
    chunks_per_thread = -(-(-(-units // C) * U * cpr) // T)
    assert chunks_per_thread * V * 2 * 12 * 32 < 2 ** 31


@pytest.mark.parametrize("dims", [[256, 256], [512, 512], [200, 200], [8192, 4], [1024, 32], [96, 96],
                                  [64, 64, 16], [40, 40, 40], [128, 64, 8], [16, 16, 128], [640, 640]])
def test_cluster_geometry(dims):
    sizes = cluster_sizes(dims)
    assert sizes, dims
    for C, V, T, slab in sizes:
        check_geometry(dims, C, V, T, slab)
