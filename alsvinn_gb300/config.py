"""Reader of alsvinn's XML run configurations: the inputs of alsvinncli
(an <fvm> section) and alsuqcli (an <fvm> plus a <uq> section).

Follows alsfvm/src/config/SimulatorSetup.cpp:102-560 and
alsuq/src/config/Setup.cpp:69-347:
  * every child of <fvm> must be one of the supported options
    (SimulatorSetup.cpp:121-131), else "Unsupported configuration option";
  * grid corners and dimension are three space-separated numbers
    (SimulatorSetup.cpp:69-79, 246-275); boundary is periodic or neumann;
  * cfl "auto" is 0.9 with reconstruction none, else 0.475; integrator
    "auto" is forwardeuler with reconstruction none, else rungekutta2
    (SimulatorSetup.cpp:294-326);
  * equationParameters.gamma sets the Euler gamma (default 1.4) and every
    equation parameter is also an initial-data parameter
    (SimulatorSetup.cpp:449-458, 487-508);
  * initialData needs a <python> file relative to the XML file; its
    <parameters> have a name, a length and one <value> (length 1) or a
    <values> list, a single value repeated to the length
    (SimulatorSetup.cpp:328-345, 459-485);
  * the writer has a type, a basename, numberOfSaves and an optional
    writeInitialTimestep; save k (1-based) is at k * endTime / numberOfSaves
    (SimulatorSetup.cpp:347-380);
  * <uq>: samples, optional sampleStart, generator ("auto" is stlmersenne),
    parameters (name, length, type, optional lower / upper / a / b), stats
    (meanvar, or structure_cube with p and numberOfH; numberOfSaves, optional
    writeInitialTimestep, writer type and basename) (Setup.cpp:69-347,
    alsuq/src/stats/StructureCube.cpp:23-31).
Platform strings cpu, cuda and gb300 all run on the GB300 path.
"""
import os
import xml.etree.ElementTree as ET
from dataclasses import dataclass, field
from typing import Dict, List, Optional

SUPPORTED_FVM_NODES = {
    "name", "platform", "boundary", "flux", "endTime", "equation", "equationParameters",
    "reconstruction", "cfl", "integrator", "initialData", "writer", "grid", "diffusion",
    "functionals",
}
PLATFORMS = ("cpu", "cuda", "gb300")
# alsuq statistics (REGISTER_STATISTICS in alsuq/src/stats/)
STATISTICS = ("meanvar", "structure_cube", "structure_basic", "functional", "onepointmoment", "bv", "bv_direction")
EQUATIONS = ("burgers", "euler1", "euler2", "euler3")
PRIMITIVE_VARIABLES = {
    "burgers": ("u",),
    "euler1": ("rho", "ux", "p"),
    "euler2": ("rho", "ux", "uy", "p"),
    "euler3": ("rho", "ux", "uy", "uz", "p"),
}
CONSERVED_VARIABLES = {
    "burgers": ("u",),
    "euler1": ("rho", "mx", "E"),
    "euler2": ("rho", "mx", "my", "E"),
    "euler3": ("rho", "mx", "my", "mz", "E"),
}


class ConfigError(RuntimeError):
    """A configuration the reference rejects, or one this library does not run."""


@dataclass
class WriterConfig:
    type: str
    basename: str
    number_of_saves: int
    write_initial_timestep: bool = False

    def save_fractions(self):
        """The writer's time coordinate: (k + 1) / numberOfSaves, with a
        leading 0 when the initial state is written (SimulatorSetup.cpp:359-363)."""
        t = [0.0] if self.write_initial_timestep else []
        return t + [(k + 1) / self.number_of_saves for k in range(self.number_of_saves)]


@dataclass
class FvmConfig:
    name: str
    platform: str
    lower: tuple
    upper: tuple
    dimension: tuple
    boundary: str
    flux: str
    end_time: float
    equation: str
    gamma: float
    reconstruction: str
    cfl: float
    integrator: str
    python_file: str
    python_program: str
    init_parameters: Dict[str, List[float]]
    writer: Optional[WriterConfig]
    diffusion: str = "none"
    functionals: List["FunctionalConfig"] = field(default_factory=list)

    @property
    def dim(self):
        return 3 if self.dimension[2] > 1 else (2 if self.dimension[1] > 1 else 1)

    def save_interval(self):
        """FixedIntervalWriter's interval endTime / numberOfSaves, 0 without a writer."""
        if self.writer is None or self.writer.number_of_saves <= 0:
            return 0.0
        return self.end_time / self.writer.number_of_saves


@dataclass
class UQParameter:
    name: str
    length: int
    type: str
    lower: float = 0.0
    upper: float = 1.0
    a: float = 0.0
    b: float = 1.0


@dataclass
class FunctionalConfig:
    """A functional and its parameters, read from a <functional> node of
    <fvm><functionals> or from a functional statistic's node, with the
    reference's parameter names (alsfvm/src/functional/*.cpp constructors)."""
    name: str
    degree: int = 0
    min_value: float = 0.0
    max_value: float = 1.0
    variables: str = ""
    gamma: float = 1.4
    p: float = 1.0
    number_of_h: int = 1
    number_of_saves: int = 0
    writer: Optional["WriterConfig"] = None

    def params(self):
        return dict(degree=self.degree, min_value=self.min_value, max_value=self.max_value,
                    variables=self.variables, gamma=self.gamma, p=self.p, number_of_h=self.number_of_h)


FUNCTIONALS = ("identity", "moment", "legendre_pointwise", "log_entropy", "bv", "structure_cube")


def _functional(node, name, gamma=None):
    """FunctionalConfig of `name` from `node`; each functional reads the
    parameters its constructor reads (missing ones raise, as
    Parameters::get* throws)."""
    if name not in FUNCTIONALS:
        raise ConfigError("Unknown functional: %s (supported: %s)" % (name, ", ".join(FUNCTIONALS)))
    f = FunctionalConfig(name=name)
    if name in ("moment", "legendre_pointwise", "bv"):
        f.degree = int(_text(node, "degree"))
    if name == "legendre_pointwise":
        f.min_value = float(_text(node, "minValue"))
        f.max_value = float(_text(node, "maxValue"))
        f.variables = _text(node, "variables", default="", required=False) or ""
    if name == "log_entropy":
        g = _text(node, "gamma", required=False)
        if g is None and gamma is None:
            raise ConfigError("log_entropy needs gamma")
        f.gamma = float(g) if g is not None else float(gamma)
    if name == "structure_cube":
        f.p = float(_text(node, "p"))
        f.number_of_h = int(_text(node, "numberOfH"))
    return f


@dataclass
class StatConfig:
    name: str
    number_of_saves: int
    write_initial_timestep: bool
    writer: WriterConfig
    p: float = 2.0          # structure_cube: the exponent; onepointmoment, bv, bv_direction: the power
    number_of_h: int = 1    # structure_cube: distances 0 .. numberOfH - 1
    functional: Optional["FunctionalConfig"] = None  # the functional statistic's functional
    direction: int = 0      # structure_basic: the axis

    def output_names(self):
        """The statistic's output names (getStatisticsNames): MeanVariance
        gives mean and variance, StructureCube "structure_cube_" plus p as
        std::to_string prints a double (StructureBasic likewise), OnePointMoment "m<p>", BoundedVariation
        "bv_<p>", BoundedVariationDirection "bv_x_<p>", "bv_y_<p>", "bv_z_<p>",
        FunctionalStatistics "mean_<functionalName>"
        (alsuq/src/stats/*.cpp constructors)."""
        if self.name == "meanvar":
            return ["mean", "variance"]
        if self.name == "structure_cube":
            return ["structure_cube_%.6f" % self.p]
        if self.name == "structure_basic":
            return ["structure_basic_%.6f" % self.p]
        if self.name == "onepointmoment":
            return ["m%d" % int(self.p)]
        if self.name == "bv":
            return ["bv_%d" % int(self.p)]
        if self.name == "bv_direction":
            return ["bv_%s_%d" % (d, int(self.p)) for d in "xyz"]
        return ["mean_" + self.functional.name]

    def save_interval(self, end_time):
        return end_time / self.number_of_saves if self.number_of_saves > 0 else 0.0


@dataclass
class UQConfig:
    samples: int
    sample_start: int
    generator: str
    parameters: List[UQParameter]
    stats: List[StatConfig] = field(default_factory=list)


@dataclass
class RunConfig:
    fvm: FvmConfig
    uq: Optional[UQConfig]
    base_path: str
    source: str


def _text(node, path, default=None, required=True):
    child = node.find(path)
    if child is None or child.text is None:
        if required and default is None:
            raise ConfigError("Missing configuration node: %s" % path)
        return default
    return child.text.strip()


def _vector(text, kind):
    parts = text.split()
    if len(parts) < 3:
        raise ConfigError("Expected three numbers, got '%s'" % text)
    return tuple(kind(p) for p in parts[:3])


def _bool(text):
    t = text.strip().lower()
    if t in ("1", "true"):
        return True
    if t in ("0", "false"):
        return False
    raise ConfigError("Not a boolean: '%s'" % text)


def _writer(node, default_saves=None):
    if node is None:
        return None
    saves = _text(node, "numberOfSaves", required=False)
    if saves is None:
        if default_saves is None:
            raise ConfigError("Missing configuration node: writer.numberOfSaves")
        saves = default_saves
    wit = _text(node, "writeInitialTimestep", required=False)
    return WriterConfig(type=_text(node, "type"), basename=_text(node, "basename"), number_of_saves=int(saves),
                        write_initial_timestep=_bool(wit) if wit is not None else False)


def _init_parameters(fvm, eq_params):
    params = {}
    # every equation parameter is also an initial-data parameter (a scalar)
    for k, v in eq_params.items():
        try:
            params[k] = [float(v)]
        except ValueError:
            params[k] = [0.0]
    node = fvm.find("initialData/parameters")
    if node is not None:
        for p in node.findall("parameter"):
            name = _text(p, "name")
            length = int(_text(p, "length"))
            if length == 1:
                values = [float(_text(p, "value"))]
            else:
                vals = p.find("values")
                values = [float(v.text) for v in (vals if vals is not None else []) if v.tag.lower() == "value"]
                if len(values) == 1:
                    values = values * length
            params[name] = values
    return params


def read_fvm(root, base_path):
    fvm = root.find("fvm")
    if fvm is None:
        raise ConfigError("Missing configuration node: fvm")
    for child in fvm:
        if child.tag not in SUPPORTED_FVM_NODES:
            raise ConfigError("Unsupported configuration option %s" % child.tag)
    lower = _vector(_text(fvm, "grid/lowerCorner"), float)
    upper = _vector(_text(fvm, "grid/upperCorner"), float)
    dimension = _vector(_text(fvm, "grid/dimension"), int)
    boundary = _text(fvm, "boundary")
    if boundary not in ("periodic", "neumann"):
        raise ConfigError("Unknown boundary conditions %s" % boundary)
    platform = _text(fvm, "platform")
    if platform not in PLATFORMS:
        raise ConfigError("Unknown platform %s (supported: %s)" % (platform, ", ".join(PLATFORMS)))
    equation = _text(fvm, "equation")
    if equation not in EQUATIONS:
        raise ConfigError("Unknown equation %s" % equation)
    reconstruction = _text(fvm, "reconstruction")
    cfl_text = _text(fvm, "cfl")
    cfl = (0.9 if reconstruction == "none" else 0.475) if cfl_text == "auto" else float(cfl_text)
    integrator = _text(fvm, "integrator")
    if integrator == "auto":
        integrator = "forwardeuler" if reconstruction == "none" else "rungekutta2"
    eq_params = {}
    epn = fvm.find("equationParameters")
    if epn is not None:
        for c in epn:
            eq_params[c.tag] = (c.text or "").strip()
    gamma = 1.4
    if equation.startswith("euler") and "gamma" in eq_params:
        gamma = float(eq_params["gamma"])
    if fvm.find("initialData/python") is None:
        raise ConfigError("Unknown initial data.")
    python_file = os.path.join(base_path, _text(fvm, "initialData/python"))
    if not os.path.exists(python_file):
        raise ConfigError("Initial data file does not exist: %s" % python_file)
    with open(python_file) as f:
        program = f.read()
    diffusion = _text(fvm, "diffusion/name", default="none", required=False)
    if diffusion != "none":
        raise ConfigError("Diffusion operator '%s' is not supported by the GB300 path (only 'none')" % diffusion)
    # <functionals><functional>: name, the functional's parameters (plus the
    # equation parameters), a writer with numberOfSaves, and numberOfSaves
    # for the FixedIntervalWriter around the IntervalFunctionalWriter
    # (SimulatorSetup::createFunctionals, SimulatorSetup.cpp:554-650)
    functionals = []
    fnode = fvm.find("functionals")
    for fn in (fnode if fnode is not None else []):
        if fn.find("time") is not None:
            raise ConfigError("Time-integrated functionals (time, timeRadius) are not supported by the GB300 path")
        saves = _text(fn, "numberOfSaves", required=False)
        if saves is None:
            raise ConfigError("Unknown arguments for functional")
        f = _functional(fn, _text(fn, "name"), gamma=gamma)
        f.number_of_saves = int(saves)
        f.writer = _writer(fn.find("writer"))
        if f.writer is None:
            raise ConfigError("Missing configuration node: writer.type")
        if f.writer.type not in ("netcdf", "numpy"):
            raise ConfigError("Unknown writer type %s (supported: netcdf, numpy)" % f.writer.type)
        functionals.append(f)
    writer = _writer(fvm.find("writer"))
    if writer is not None and writer.type not in ("netcdf", "numpy"):
        raise ConfigError("Unknown writer type %s (supported: netcdf, numpy)" % writer.type)
    return FvmConfig(name=_text(fvm, "name"), platform=platform, lower=lower, upper=upper, dimension=dimension,
                     boundary=boundary, flux=_text(fvm, "flux"), end_time=float(_text(fvm, "endTime")),
                     equation=equation, gamma=gamma, reconstruction=reconstruction, cfl=cfl,
                     integrator=integrator, python_file=python_file, python_program=program,
                     init_parameters=_init_parameters(fvm, eq_params), writer=writer, diffusion=diffusion,
                     functionals=functionals)


def read_uq(root):
    uq = root.find("uq")
    if uq is None:
        return None
    generator = _text(uq, "generator", default="auto", required=False)
    if generator == "auto":
        generator = "stlmersenne"
    if generator != "stlmersenne":
        raise ConfigError("Unknown generator %s (supported: stlmersenne)" % generator)
    params = []
    pnode = uq.find("parameters")
    for p in (pnode if pnode is not None else []):
        typ = _text(p, "type")
        if typ == "normal":
            raise ConfigError("Normal variables are not supported in the current implementation."
                              " Use Uniform and scipy.stats.norm.ppf(X) where X is the random viriable.")
        if typ not in ("uniform", "uniform1d"):
            raise ConfigError("Unknown distribution %s (supported: uniform, uniform1d)" % typ)
        # Setup::makeSampleGenerator puts lower = 0, upper = 1, a = 0, b = 1
        # into the parameter's tree after reading it (Setup.cpp:172-181;
        # ptree::put replaces an existing value), so values given in the XML
        # never reach the distribution: the defaults are kept here as well
        params.append(UQParameter(name=_text(p, "name"), length=int(_text(p, "length")), type=typ))
    stats = []
    snode = uq.find("stats")
    for s in (snode if snode is not None else []):
        name = _text(s, "name")
        if name not in STATISTICS:
            raise ConfigError("Unknown statistics %s (supported: %s)" % (name, ", ".join(STATISTICS)))
        saves = _text(s, "numberOfSaves", required=False)
        if saves is None:
            raise ConfigError("Statistics %s needs numberOfSaves (time-integrated statistics are not supported)"
                              % name)
        wit = _text(s, "writeInitialTimestep", required=False)
        extra = {}
        if name == "structure_cube":
            extra = dict(p=float(_text(s, "p")), number_of_h=int(_text(s, "numberOfH")))
        elif name == "structure_basic":
            extra = dict(p=float(_text(s, "p")), number_of_h=int(_text(s, "numberOfH")),
                         direction=int(_text(s, "direction")))
        elif name in ("onepointmoment", "bv", "bv_direction"):
            extra = dict(p=float(int(_text(s, "p"))))
        elif name == "functional":
            extra = dict(functional=_functional(s, _text(s, "functionalName")))
        stats.append(StatConfig(name=name, number_of_saves=int(saves),
                                write_initial_timestep=_bool(wit) if wit is not None else False,
                                writer=_writer(s.find("writer"), default_saves=saves), **extra))
    return UQConfig(samples=int(float(_text(uq, "samples"))),
                    sample_start=int(_text(uq, "sampleStart", default="0", required=False)),
                    generator=generator, parameters=params, stats=stats)


def read_config(filename):
    """Parses an alsvinn XML input; raises ConfigError as the reference
    throws."""
    if not os.path.exists(filename):
        raise ConfigError("Input file does not exist\n%s" % filename)
    base = os.path.dirname(os.path.abspath(filename))
    with open(filename) as f:
        text = f.read()
    try:
        root = ET.fromstring(text)
    except ET.ParseError as e:
        raise ConfigError("XML parse error in %s: %s" % (filename, e))
    if root.tag != "config":
        raise ConfigError("Missing configuration node: config")
    return RunConfig(fvm=read_fvm(root, base), uq=read_uq(root), base_path=base, source=text)
