"""Initial data from the reference's Python programs, evaluated on the host.

alsfvm's PythonInitialData (alsfvm/src/init/PythonInitialData.cpp:84-281)
runs the program of the XML's <initialData><python> file in an embedded
interpreter, in one of two forms:

  * snippet: the program is the body of
        def initial_data(x, y, z, i, j, k, output):
    with every primitive variable (rho, ux, uy, uz, p or u) preset to 0.0 and
    copied to output[name] at the end; it is called once per interior cell
    at the cell midpoint, in z, y, x loop order;
  * global: a program defining init_global(<var>_global..., nx, ny, nz, ax,
    ay, az, bx, by, bz) (detected by the text "init_global"), called once with
    writable arrays of shape (nx, ny, nz), x varying fastest in memory.

The namespace starts with `from math import *` and then, when numpy imports,
`from numpy import *`; parameters (from the XML and from the UQ generator)
are globals, as Python floats (length 1) or float64 arrays. This module
evaluates the same program text the same way in this process's interpreter,
which is what makes the values identical to the reference's.
"""
import numpy as np

from .config import PRIMITIVE_VARIABLES


class InitialDataError(RuntimeError):
    pass


def cell_midpoints(lower, upper, dimension):
    """Midpoints per axis as Grid::getCellMidpoints forms them
    (alsfvm/src/grid/Grid.cpp:24-42, 148-165): origin + length * i +
    length / 2, the length of an inactive y or z axis being 1."""
    out = []
    for d in range(3):
        n = dimension[d]
        h = (upper[d] - lower[d]) / n
        if d > 0 and n == 1:
            h = 1.0
        out.append([lower[d] + h * i + h / 2.0 for i in range(n)])
    return out


def _namespace(parameters):
    ns = {"__name__": "__alsvinn_initial_data__"}
    exec("from math import *", ns)
    try:
        exec("from numpy import *", ns)
    except ImportError:
        pass
    for name, value in (parameters or {}).items():
        v = list(value)
        ns[name] = float(v[0]) if len(v) == 1 else np.array(v, dtype=np.float64)
    return ns


def _indent(program):
    return "".join("    " + line + "\n" for line in program.splitlines())


def evaluate(program, equation, lower, upper, dimension, parameters=None):
    """Primitive variables of the interior cells: array (nvar, nz, ny, nx)."""
    names = PRIMITIVE_VARIABLES[equation]
    nx, ny, nz = dimension
    prim = np.zeros((len(names), nz, ny, nx))
    ns = _namespace(parameters)
    try:
        if "init_global" in program:
            exec(program, ns)
            views = [prim[v].transpose(2, 1, 0) for v in range(len(names))]  # (nx, ny, nz), x fastest
            ns["init_global"](*views, nx, ny, nz, lower[0], lower[1], lower[2], upper[0], upper[1], upper[2])
        else:
            src = "def initial_data(x, y, z, i, j, k, output):\n"
            src += "".join("    %s = 0.0\n" % n for n in names)
            src += _indent(program)
            src += "".join("    output['%s'] = %s\n" % (n, n) for n in names)
            exec(src, ns)
            fn = ns["initial_data"]
            xs, ys, zs = cell_midpoints(lower, upper, dimension)
            out = {}
            for k in range(nz):
                for j in range(ny):
                    for i in range(nx):
                        fn(xs[i], ys[j], zs[k], i, j, k, out)
                        for v, n in enumerate(names):
                            prim[v, k, j, i] = float(out[n])
    except Exception as e:
        raise InitialDataError("Error in the initial data program: %s: %s" % (type(e).__name__, e)) from e
    return prim
