"""Generate golden vectors by running the reference lightprop2d 1.0.4 itself.

Run where the reference source is available, giving its checkout path::

    python tests/golden/make_golden.py <path of the lightprop2d 1.0.4 checkout>

It imports the reference unchanged.  The one shim it needs is a stand-in for
``cp.ndarray``: beam2d.py:135 annotates ``cp.ndarray`` even when cupy is absent,
which raises NameError at import.  Defining ``builtins.cp`` with a dummy
``ndarray`` type lets the import succeed; cupy stays unused (``_using_cupy`` is
False) and profiles.py falls back to numpy.

The output, ``golden.npz``, is committed; nothing on the GPU side reads the
reference at run time.
"""
import builtins
import os
import sys
import types
import warnings

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def import_reference(path):
    builtins.cp = types.SimpleNamespace(ndarray=type("ndarray", (), {}))
    sys.path.insert(0, path)
    warnings.simplefilter("ignore")
    import lightprop2d  # noqa: E402
    return lightprop2d


def main(ref_path):
    lp = import_reference(ref_path)
    sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
    from oracle.lp_oracle import random_phase_hole

    um, nm, mm = lp.um, lp.nm, lp.mm
    out = {}

    # --- 256^2 / 200 um / 632 nm random amplitude+phase hole (r = 25 um),
    #     complex128, propagate(100 um) once, then iprofile.
    f0 = random_phase_hole(256, 200 * um, 25 * um, seed=20240601)
    b = lp.Beam2D(200 * um, 256, 632 * nm, init_field=f0.copy())
    b.propagate(100 * um)
    out["cfg1_seed"] = np.array(20240601)
    out["cfg1_in_abs_sum"] = np.array(np.abs(f0).sum())
    out["cfg1_field"] = b.field
    out["cfg1_iprofile"] = b.iprofile.astype(np.float32)

    # --- Gaussian, sequential propagates (spectrum is state, z accumulates).
    g = lp.Beam2D(2 * mm, 64, 632 * nm, init_field_gen=lp.gaussian_beam,
                  init_gen_args=(1, 100 * um))
    out["seq_in"] = g.field.copy()
    for i, dz in enumerate([0.1, 0.9, 4.0]):
        g.propagate(dz)
        out[f"seq_field_{i}"] = g.field.copy()
        out[f"seq_spectrum_{i}"] = g.spectrum.copy()
    out["seq_z"] = np.array(g.z)

    # --- lens then propagate (the lens sign/scale convention: k0 = 1/wl, e^{+i phi}).
    L = lp.Beam2D(500 * um, 64, 532 * nm, init_field_gen=lp.gaussian_beam,
                  init_gen_args=(1, 50 * um))
    out["lens_in"] = L.field.copy()
    L.lens(-0.1)
    out["lens_field"] = L.field.copy()
    out["lens_spectrum"] = L.spectrum.copy()
    L.propagate(0.02)
    out["lens_prop_field"] = L.field.copy()
    out["lens_prop_spectrum"] = L.spectrum.copy()

    # --- filters: generator masks and array masks on both grids.
    rng = np.random.default_rng(7)
    xmask = rng.uniform(0.5, 1.0, size=(64, 64))
    kmask = rng.uniform(0.5, 1.0, size=(64, 64)) * np.exp(
        2j * np.pi * rng.uniform(size=(64, 64)))
    F = lp.Beam2D(200 * um, 64, 632 * nm, init_field_gen=lp.gaussian_beam,
                  init_gen_args=(1, 40 * um))
    out["filt_in"] = F.field.copy()
    F.coordinate_filter(f_gen=lp.round_hole, fargs=(50 * um,))
    out["filt_cf_gen_field"] = F.field.copy()
    F.coordinate_filter(f_init=xmask)
    out["filt_cf_arr_field"] = F.field.copy()
    out["filt_cf_arr_spectrum"] = F.spectrum.copy()
    F.spectral_filter(f_gen=lambda kx, ky, s: np.exp(-(kx ** 2 + ky ** 2) / s ** 2),
                      fargs=(2000.0,))
    out["filt_sf_gen_field"] = F.field.copy()
    F.spectral_filter(f_init=kmask)
    out["filt_sf_arr_field"] = F.field.copy()
    out["filt_sf_arr_spectrum"] = F.spectrum.copy()
    F.propagate(0.05)
    out["filt_prop_field"] = F.field.copy()
    out["filt_xmask"] = xmask
    out["filt_kmask"] = kmask

    # --- evanescent components: Nyquist (16000 /cm) exceeds k0 (15823 /cm).
    E = lp.Beam2D(20 * um, 64, 632 * nm, init_field_gen=lp.gaussian_beam,
                  init_gen_args=(1, 3 * um))
    out["evan_in"] = E.field.copy()
    out["evan_fraction"] = np.array(np.mean(E.Kz == 0))
    E.propagate(5 * um)
    out["evan_field"] = E.field.copy()

    # --- negative z returns to the start; z == 0 is a no-op.
    Z = lp.Beam2D(1 * mm, 64, 1064 * nm, init_field_gen=lp.gaussian_beam,
                  init_gen_args=(1, 60 * um))
    out["negz_in"] = Z.field.copy()
    Z.propagate(0.3)
    out["negz_fwd"] = Z.field.copy()
    Z.propagate(0)
    out["negz_zero"] = Z.field.copy()
    Z.propagate(-0.3)
    out["negz_back"] = Z.field.copy()
    out["negz_z"] = np.array(Z.z)

    # --- complex64 reference path (the complex128 transfer function is cast
    #     into the complex64 spectrum by the in-place multiply).
    C = lp.Beam2D(2 * mm, 64, 632 * nm, init_field_gen=lp.gaussian_beam,
                  init_gen_args=(1, 100 * um), complex_bits=64)
    C.propagate(1.0)
    out["c64_field"] = C.field.copy()
    out["c64_dtype_ok"] = np.array(C.field.dtype == np.complex64)

    # --- init_spectrum independent of init_field: propagate uses the spectrum.
    rng = np.random.default_rng(11)
    fa = rng.normal(size=(64, 64)) + 1j * rng.normal(size=(64, 64))
    sb = np.fft.fft2(rng.normal(size=(64, 64)) + 1j * rng.normal(size=(64, 64)))
    # beam2d.py:133 stores init_spectrum without a copy and propagate then
    # multiplies it in place, so hand the reference its own copy.
    S = lp.Beam2D(300 * um, 64, 800 * nm, init_field=fa, init_spectrum=sb.copy())
    S.propagate(0.01)
    out["ispec_field_in"] = fa
    out["ispec_spectrum_in"] = sb
    out["ispec_field"] = S.field.copy()

    # --- mixed sequence of every operation on the path.
    Q = lp.Beam2D(400 * um, 64, 700 * nm, init_field_gen=lp.gaussian_beam,
                  init_gen_args=(1, 30 * um))
    out["mix_in"] = Q.field.copy()
    Q.lens(2.0)
    Q.propagate(0.5)
    Q.coordinate_filter(f_gen=lp.square_hole, fargs=(150 * um,))
    Q.propagate(0.25)
    Q.spectral_filter(f_init=kmask)
    Q.propagate(-0.1)
    out["mix_field"] = Q.field.copy()
    out["mix_spectrum"] = Q.spectrum.copy()
    out["mix_z"] = np.array(Q.z)

    # --- profile generators on a 32x32 grid (profiles.py).
    n, dL = 32, 1e-4
    x = np.arange(-n // 2, n // 2, 1) * dL
    y = x.reshape((-1, 1))
    out["prof_plane"] = lp.plane_wave(x.copy(), y.copy())
    out["prof_gauss"] = lp.gaussian_beam(x.copy(), y.copy(), 1.5, 8 * dL, dL, -2 * dL)
    out["prof_round"] = lp.round_hole(x.copy(), y.copy(), 8 * dL, 2 * dL, 0)
    out["prof_rect"] = lp.rectangle_hole(x.copy(), y.copy(), 10 * dL, 6 * dL, dL, 0)
    out["prof_square"] = lp.square_hole(x.copy(), y.copy(), 8 * dL)
    out["prof_slits"] = lp.square_slits(x.copy(), y.copy(), 4 * dL, 10 * dL)
    np.random.seed(5)
    out["prof_rand_round"] = lp.random_round_hole(x.copy(), y.copy(), 8 * dL)
    np.random.seed(5)
    out["prof_rand_round_bin"] = lp.random_round_hole_bin(x.copy(), y.copy(), 8 * dL, 0, 0, 2)
    np.random.seed(5)
    out["prof_rand_round_phase"] = lp.random_round_hole_phase(x.copy(), y.copy(), 8 * dL)

    # --- analytic Gaussian known-answer inputs (tests/test_analytics.py:53-71 setup).
    for tag, R in (("a8", 3 * mm / 8), ("a16", 3 * mm / 16)):
        K = lp.Beam2D(3 * mm, 512, 632 * nm, init_field_gen=lp.gaussian_beam,
                      init_gen_args=(1, R))
        zs = np.arange(20) * 0.02
        K.propagate(zs[0])
        vals = []
        for _ in zs:
            vals.append(K.iprofile[256, 256])
            K.propagate(0.02)
        out[f"kat_{tag}_R"] = np.array(R)
        out[f"kat_{tag}_I"] = np.array(vals)
        out[f"kat_{tag}_k0"] = np.array(K.k0)

    # --- beam metrics (beam2d.py:669-752): centroid, D4sigma, centroid_intensity.
    def metrics(beam):
        Xc, Yc, nxc, nyc = beam.centroid
        dx, dy = beam.D4sigma
        return np.array([Xc, Yc, nxc, nyc, dx, dy, beam.centroid_intensity])

    out["met_cfg1"] = metrics(b)
    M = lp.Beam2D(1 * mm, 512, 632 * nm, init_field_gen=lp.gaussian_beam,
                  init_gen_args=(1, 50 * um, 200 * um, -150 * um), complex_bits=64)
    out["met_off_in"] = metrics(M)
    M.lens(3.0)
    M.propagate(2.0)
    out["met_off_prop"] = metrics(M)

    # --- grid management (beam2d.py:375-460): expand (edge replication) and
    #     coarse (block mean); each ends with a new FFT.  crop needs
    #     scipy.interpolate.interp2d, removed from SciPy >= 1.14.
    G = lp.Beam2D(1 * mm, 128, 632 * nm, init_field_gen=lp.gaussian_beam,
                  init_gen_args=(1, 150 * um, 100 * um, 0), complex_bits=64)
    G.propagate(1.0)
    out["grid_in"] = G.field.copy()
    G.expand(2 * mm)
    out["grid_expand_n"] = np.array(G.npoints)
    out["grid_expand_field"] = G.field.copy()
    out["grid_expand_spectrum"] = G.spectrum.copy()
    G.coarse(2)
    out["grid_coarse_n"] = np.array(G.npoints)
    out["grid_coarse_field"] = G.field.copy()
    out["grid_coarse_spectrum"] = G.spectrum.copy()
    try:
        G.crop(0.5 * mm)
        out["grid_crop_runs"] = np.array(True)
    except Exception as e:  # interp2d is gone from current SciPy
        out["grid_crop_runs"] = np.array(False)
        out["grid_crop_error"] = np.array(type(e).__name__)

    # --- mode decomposition (beam2d.py:539-667) with a synthetic complex
    #     Hermite-Gauss-like basis on a 32x32 window of a 64x64 beam.
    nb, w = 32, 6 * um
    xb = (np.arange(nb) - nb / 2 + 0.5) * (1.5 * um)
    XB, YB = np.meshgrid(xb, xb)
    herm = [np.ones_like(xb), 2 * xb / w, 4 * (xb / w) ** 2 - 2, 8 * (xb / w) ** 3 - 12 * xb / w]
    modes = []
    for a_ in range(4):
        for b_ in range(4 - a_):
            mm = np.outer(herm[b_], herm[a_]) * np.exp(-(XB ** 2 + YB ** 2) / w ** 2)
            mm = mm * np.exp(1j * 0.37 * (a_ + 2 * b_))
            modes.append((mm / np.linalg.norm(mm)).ravel())
    modes = np.array(modes)
    Q = lp.Beam2D(96 * um, 64, 1064 * nm, init_field_gen=lp.gaussian_beam,
                  init_gen_args=(1, 8 * um, 2 * um, -1 * um))
    Q.propagate(50 * um)
    out["modes_basis"] = modes
    out["modes_field"] = Q.field.copy()
    out["modes_scalar"] = Q.deconstruct_by_modes(modes)
    out["modes_lstsq"] = Q.deconstruct_by_modes(modes, "lstsq")
    mt = np.vstack(modes).T
    out["modes_fast"] = Q.fast_deconstruct_by_modes(mt.T, mt.T.dot(mt))
    Q.construct_by_modes(modes, out["modes_scalar"] * np.exp(0.5j))
    out["modes_constructed"] = Q.field.copy()
    out["modes_constructed_spectrum"] = Q.spectrum.copy()

    # --- config 2 at its full size: Gaussian 2048^2, area 2 mm, 632 nm,
    #     waist 100 um, complex128, propagate(1 cm) then propagate(9 cm)
    #     (z = 10 cm).  Kept small: the central 64^2 window, every 16th point
    #     of the centre row and column, and the total energy.
    W = lp.Beam2D(2 * lp.mm, 2048, 632 * lp.nm, init_field_gen=lp.gaussian_beam,
                  init_gen_args=(1, 100 * lp.um))
    for tag, dz in (("z1", 1.0), ("z10", 9.0)):
        W.propagate(dz)
        f = W.field
        out[f"cfg2_{tag}_window"] = f[992:1056, 992:1056].copy()
        out[f"cfg2_{tag}_row"] = f[1024, ::16].copy()
        out[f"cfg2_{tag}_col"] = f[::16, 1024].copy()
        out[f"cfg2_{tag}_energy"] = np.array(np.sum(np.abs(f) ** 2))

    # --- sizes that are not powers of two (the reference takes any npoints):
    #     even 100 and odd 75; lens then propagate, a coordinate and a
    #     spectral filter, the spectrum and iprofile.
    for n, tag in ((100, "np100"), (75, "np75")):
        V = lp.Beam2D(1 * lp.mm, n, 632 * lp.nm, init_field_gen=lp.gaussian_beam,
                      init_gen_args=(1, 150 * lp.um))
        out[f"{tag}_in"] = V.field.copy()
        V.lens(5.0)
        V.propagate(0.3)
        out[f"{tag}_lens_prop_field"] = V.field.copy()
        out[f"{tag}_lens_prop_spectrum"] = V.spectrum.copy()
        V.coordinate_filter(f_gen=lp.round_hole, fargs=(300 * lp.um,))
        V.spectral_filter(f_gen=lp.gaussian_beam, fargs=(1, 2e4))
        V.propagate(0.5)
        out[f"{tag}_filt_prop_field"] = V.field.copy()
        out[f"{tag}_filt_prop_iprofile"] = V.iprofile.copy()
        out[f"{tag}_z"] = np.array(V.z)

    np.savez_compressed(os.path.join(HERE, "golden.npz"), **out)
    print("wrote", len(out), "arrays")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <path of the lightprop2d checkout>")
    main(sys.argv[1])
