# Sod shock tube on the whole grid at once (init_global form)
def init_global(rho, ux, p, nx, ny, nz, ax, ay, az, bx, by, bz):
    h = (bx - ax) / nx
    x = ax + h * arange(nx) + h / 2.0
    left = x < 0.0
    rho[:, 0, 0] = where(left, 1.0, 0.125)
    ux[:, 0, 0] = 0.0
    p[:, 0, 0] = where(left, 1.0, 0.1)
