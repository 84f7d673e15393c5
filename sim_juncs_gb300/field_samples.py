"""The monitor output file of bound_geom::save_field_times (src/disp.cpp:758-923),
from the samples and spectra the stepper keeps on the device.

The tree is the reference's ``field_samples.h5`` layout, path for path:

  info/time_bounds            [3]  {0, ttot in fs, step in fs}    (:820-825)
  info/n_clusters             [1]  number of monitor clusters     (:826-831)
  info/n_time_points          [1]  n_t_pts / save_span            (:832-836)
  info/sources                [n]  {wavelen, width, phase, start_time,
                                    end_time, amplitude}          (:786-793, :837-847)
  info/cgs_params/<name>      [1]  every numeric CGS variable     (:848-862)
  cluster_<k>/locations       [m]  {x, y, z}                      (:886-895)
  cluster_<k>/point_<i>/time       {Re, Im}                       (:900-917)
  cluster_<k>/point_<i>/frequency  {Re, Im}

with the reference's own quirks kept, since readers of its files rely on
them:

  * the time datasets hold n_t_pts // save_span samples (the dataspace of
    :772), although the loop records ceil(n_t_pts / save_span) (:721): when
    save_span does not divide n_t_pts the last sample is left out; the
    frequency datasets are the fft (src/data_utils.cpp:413-427) of every
    recorded sample, all of them as long as the last monitor's (:809);
  * one cluster more than n_clusters is written (:879): cluster_<n_clusters>
    holds the points after the last cluster's end, usually none, with an
    empty locations dataset;
  * cluster numbers have floor(log10(n_clusters)) + 1 digits and point
    numbers floor(log10(n_points)) + 1 digits, zero padded (write_number,
    src/argparse.h:58-80); point numbers run over all monitors, not per
    cluster.

``write`` stores the tree as HDF5 when h5py is importable, with the
compound types above, and otherwise as an .npz archive whose keys are the
same paths (structured arrays for the compound types).
"""
import math

import numpy as np

LIGHT_SPEED_UM_PER_FS = 0.299792458   # meep_time_to_fs, src/disp.hpp:158


def _digits(n):
    # (size_t)(log(n) / log(10)) + 1, as src/disp.cpp:872-873 computes it
    return int(math.log(n) / math.log(10)) + 1 if n > 0 else 1


def complex_dtype(real=np.float64):
    return np.dtype([("Re", real), ("Im", real)])


def location_dtype(real=np.float64):
    return np.dtype([("x", real), ("y", real), ("z", real)])


def source_dtype(real=np.float64):
    return np.dtype([(k, real) for k in ("wavelen", "width", "phase", "start_time", "end_time", "amplitude")])


def build_tree(samples, spectra, locations, clusters, ttot, n_t_pts, save_span, sources=(), cgs_params=None,
               um_scale=1.0, real=np.float64):
    """The file's datasets as {path: numpy array}.

    samples[i]   the recorded series of monitor i (ceil(n_t_pts / save_span)
                 values, real or complex)
    spectra[i]   its fft (complex)
    locations    [n_monitors][3] monitor positions (meep units)
    clusters     the cluster end indices (bound_geom::monitor_clusters)
    ttot         total simulated time (meep units), n_t_pts the step count
    sources      (wavelen, width, phase, start_time, end_time, amplitude) per source
    cgs_params   {name: number} of the scene's numeric variables
    """
    n_locs = len(samples)
    if len(spectra) != n_locs or len(locations) != n_locs:
        raise ValueError("samples, spectra and locations must have one entry per monitor")
    if save_span < 1:
        save_span = 1
    n_keep = n_t_pts // save_span
    cdt, ldt, sdt = complex_dtype(real), location_dtype(real), source_dtype(real)
    tree = {}
    t1 = ttot / (LIGHT_SPEED_UM_PER_FS * um_scale)
    tree["info/time_bounds"] = np.array([0.0, t1, (t1 - 0.0) * save_span / n_t_pts], dtype=real)
    tree["info/n_clusters"] = np.array([len(clusters)], dtype=np.uint64)
    tree["info/n_time_points"] = np.array([n_keep], dtype=np.uint64)
    src = np.zeros(len(sources), dtype=sdt)
    for q, s in enumerate(sources):
        src[q] = tuple(float(v) for v in s)
    tree["info/sources"] = src
    for name, v in (cgs_params or {}).items():
        tree[f"info/cgs_params/{name}"] = np.array([v], dtype=real)
    n_freq = len(spectra[-1]) if n_locs else 0
    locs = np.zeros(n_locs, dtype=ldt)
    for q, p in enumerate(locations):
        locs[q] = tuple(float(v) for v in p)
    gd, pd = _digits(len(clusters)), _digits(n_locs)
    start = 0
    i = 0   # point numbers run over every monitor, across clusters
    for k in range(len(clusters) + 1):
        end = n_locs if k >= len(clusters) else int(clusters[k])
        cname = f"cluster_{k:0{gd}d}"
        tree[f"{cname}/locations"] = locs[start:end].copy()
        start = end
        while i < end:
            t = np.asarray(samples[i])
            if t.size < 2:
                # src/disp.cpp:904-907 leaves the loop at such a point without
                # advancing, so no later point is written either
                break
            td = np.zeros(n_keep, dtype=cdt)
            m = min(n_keep, t.size)
            td["Re"][:m] = np.real(t[:m])
            td["Im"][:m] = np.imag(t[:m]) if np.iscomplexobj(t) else 0.0
            f = np.asarray(spectra[i])
            fd = np.zeros(n_freq, dtype=cdt)
            m = min(n_freq, f.size)
            fd["Re"][:m] = f.real[:m]
            fd["Im"][:m] = f.imag[:m]
            pname = f"{cname}/point_{i:0{pd}d}"
            tree[f"{pname}/time"] = td
            tree[f"{pname}/frequency"] = fd
            i += 1
    return tree


def from_fields(fields, ttot=None, clusters=None, inst=0, sources=(), cgs_params=None, um_scale=1.0,
                real=np.float64):
    """The tree of one instance of a sim_juncs_gb300.fields.Fields after its
    run: its monitor samples, their device spectra and its monitor probes'
    positions.  ttot defaults to the steps run times dt (n_t_pts = steps)."""
    samples = fields.monitors(inst)
    spectra = fields.monitor_spectrum(inst)
    probes = [p for p in fields.instances[inst].probes if p.monitor]
    n_t = fields.steps_done
    if ttot is None:
        ttot = n_t * fields.dt(inst)
    if clusters is None:
        clusters = [len(probes)]
    return build_tree(list(samples), list(spectra), [p.pos for p in probes], clusters, ttot, n_t,
                      fields.instances[inst].save_span, sources, cgs_params, um_scale, real)


def write(path, tree):
    """HDF5 where h5py is importable, else an .npz archive keyed by path;
    returns the file written."""
    try:
        import h5py
    except ImportError:
        h5py = None
    if h5py is not None:
        with h5py.File(path, "w") as fh:
            for key, arr in tree.items():
                fh.create_dataset(key, data=arr)
        return path
    if not path.endswith(".npz"):
        path = path + ".npz"
    np.savez(path, **tree)
    return path


def read(path):
    """{path: array} of a file written by ``write``."""
    if path.endswith(".npz"):
        with np.load(path) as z:
            return {k: z[k] for k in z.files}
    import h5py
    out = {}
    with h5py.File(path, "r") as fh:
        fh.visititems(lambda name, obj: out.__setitem__(name, obj[()]) if isinstance(obj, h5py.Dataset) else None)
    return out
