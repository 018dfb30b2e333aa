"""Host side of the standalone particle tracer (code/app/src/pic_tracer.cxx):
the configuration its ``main`` builds, the particle box and species of its map
operator, and the per-frame result files it writes. The tracing itself is
``allscale_ipic3d_gb300.trace`` (the CUDA path, ``ipic3d_gpu_trace``)."""
import os

import numpy as np

from .abi import Props

ELEMENTARY_CHARGE = 1.602176565e-19  # pic_tracer.cxx:220
PROTON_MASS = 1.672621777e-27        # pic_tracer.cxx:222
KINETIC_ENERGY = 1e7 * ELEMENTARY_CHARGE  # pic_tracer.cxx:221 (J)


def tracer_props(R=64):
    """The UniverseProperties pic_tracer's main sets up for an R^3 grid
    (pic_tracer.cxx:196-214): dt 0.01, c 299792458, Earth radius 6378137 m,
    cell width 20 R_E / R, the box centred on the planet, Bext = (0, 0,
    3.07e-5)."""
    p = Props()
    p.dt = 0.01
    p.speed_of_light = 299792458.0
    p.size[:] = [int(R)] * 3
    p.planet_radius = 6378137.0
    w = (20.0 / int(R)) * p.planet_radius
    p.cell_width[:] = [w] * 3
    p.object_center[:] = [0.0, 0.0, 0.0]
    p.origin[:] = [p.object_center[a] - int(R) * w / 2.0 for a in range(3)]
    p.external_b[:] = [0.0, 0.0, 3.07e-5]
    return p


def speed_scale(props):
    """v_mod of pic_tracer.cxx:223: the speed of a proton of kinetic energy
    10 MeV, the width of the normal velocity distribution."""
    c = props.speed_of_light
    return c / np.sqrt(1.0 + (PROTON_MASS * c * c) / KINETIC_ENERGY)


def particle_box(props):
    """[low, hig) of the uniform positions (pic_tracer.cxx:230-231): the
    middle three quarters of the universe box."""
    extent = np.array(props.cell_width) * np.array(props.size, dtype=np.float64)
    low = np.array(props.origin) + extent / 8.0
    return low, low + 0.75 * extent


def _g(v):
    """A double as the default C++ stream prints it (6 significant digits)."""
    return "%g" % v


def frame_text(counts, t, props):
    """The text of result file t (pic_tracer.cxx:292-306): a header, then
    `t,x*w,y*w,z*w,count` for every cell, x slowest."""
    sx, sy, sz = props.shape
    w = props.cell_width
    c = np.asarray(counts).reshape(-1, sx, sy, sz)[t]
    xs = [_g(x * w[0]) for x in range(sx)]
    ys = [_g(y * w[1]) for y in range(sy)]
    zs = [_g(z * w[2]) for z in range(sz)]
    lines = ["t,x,y,z,density"]
    for x in range(sx):
        for y in range(sy):
            row = c[x, y]
            pre = "%d,%s,%s," % (t, xs[x], ys[y])
            lines.extend(pre + zs[z] + "," + str(int(row[z])) for z in range(sz))
    return "\n".join(lines) + "\n"


def write_frames(counts, props, stamp, directory="."):
    """Writes result_<stamp>.csv.NNNNNN for every frame of a histogram as
    pic_tracer does (its stamp is the steady-clock time in ms). Returns the
    paths."""
    frames = np.asarray(counts).reshape(-1, props.ncells).shape[0]
    paths = []
    for t in range(frames):
        path = os.path.join(directory, "result_%d.csv.%06d" % (int(stamp), t))
        with open(path, "w") as f:
            f.write(frame_text(counts, t, props))
        paths.append(path)
    return paths
