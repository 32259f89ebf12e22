# Kelvin-Helmholtz with a seeded interface perturbation: a[0:10] weights
# (normalised) and a[10:20] phases (times 2 pi) of the lower interface,
# a[20:30] and a[30:40] of the upper one; evaluated at cell midpoints.
def init_global(rho, ux, uy, p, nx, ny, nz, ax, ay, az, bx, by, bz):
    hx = (bx - ax) / nx
    hy = (by - ay) / ny
    x = ax + hx * arange(nx) + hx / 2.0
    y = ay + hy * arange(ny) + hy / 2.0

    def bump(w, phase):
        s = w.sum()
        w = w / (s if abs(s) > 1e-10 else 1.0)
        return 0.01 * sum([w[j] * cos(2 * pi * phase[j] + 2 * pi * (j + 1) * x) for j in range(10)], 0)

    lower = 0.25 + bump(a[0:10], a[10:20])
    upper = 0.75 + bump(a[20:30], a[30:40])
    X, Y = meshgrid(x, y, indexing="ij")
    inside = (Y > lower[:, None]) & (Y < upper[:, None])
    rho[:, :, 0] = where(inside, 2.0, 1.0)
    ux[:, :, 0] = where(inside, -0.5, 0.5)
    uy[:, :, 0] = 0.0
    p[:, :, 0] = 2.5
