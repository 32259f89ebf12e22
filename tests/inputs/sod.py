# Sod shock tube, evaluated per cell midpoint (snippet form)
if x < 0.0:
    rho = 1.0
    ux = 0.0
    p = 1.0
else:
    rho = 0.125
    ux = 0.0
    p = 0.1
