"""Generate the golden vectors that pin the oracle to lentil 0.8.8 itself.

Runs lentil from its source tree (read-only) on seeded inputs and writes
small ``.npz`` fixtures next to this script.  The reference package cannot
travel to the GPU machine, so the fixtures are committed and the tests only
read them.

Usage (the argument is the root of a lentil 0.8.8 source tree, the
directory that holds its ``lentil/`` package):

    PYTHONDONTWRITEBYTECODE=1 python tests/golden/make_golden.py <lentil-source-root>
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def main(ref_root):
    sys.dont_write_bytecode = True
    sys.path.insert(0, ref_root)
    import lentil
    import lentil.field
    import lentil.fourier
    import lentil.helper
    import lentil.propagate
    import lentil.radiometry

    rng = np.random.default_rng(20261203)

    def crand(*shape):
        return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)

    # ---------------------------------------------------------------- dft2
    d = {}
    cases = [
        # name, f shape, alpha, shape, shift, offset, unitary
        ('even10', (10, 10), 1 / 10, None, (0, 0), (0, 0), False),
        ('odd11', (11, 11), 1 / 11, None, (0, 0), (0, 0), False),
        ('rect10x11', (10, 11), (1 / 10, 1 / 11), None, (0, 0), (0, 0), False),
        ('general', (23, 17), (0.013, 0.021), (31, 29), (2.3, -1.7), (3, -2), True),
        ('floatoff', (16, 20), (0.011, 0.017), (24, 18), (-3.0, 4.0), (0.5, -1.25), True),
        ('wide', (64, 64), 1 / 200, (96, 80), (0.25, -0.75), (0, 0), True),
        ('negalpha', (12, 9), (-0.05, 0.03), (13, 15), (1.0, 0.0), (-2, 1), True),
        ('big', (128, 96), (1.3e-3, 2.1e-3), (160, 144), (5.5, -7.25), (-11, 6), True),
    ]
    names = []
    for name, fs, alpha, shape, shift, offset, unitary in cases:
        f = crand(*fs)
        F = lentil.fourier.dft2(f, alpha, shape=shape, shift=shift, offset=offset,
                                unitary=unitary)
        d[f'{name}_f'] = f
        d[f'{name}_F'] = F
        d[f'{name}_alpha'] = np.broadcast_to(alpha, (2,)).astype(float)
        d[f'{name}_shape'] = np.asarray(F.shape)
        d[f'{name}_shift'] = np.asarray(shift, float)
        d[f'{name}_offset'] = np.asarray(offset, float)
        d[f'{name}_unitary'] = np.asarray(unitary)
        names.append(name)
    # integer shift moves the centroid exactly (tests/test_fourier.py:68-78)
    n = 100
    shift = np.array([7.0, -12.0])
    d['shift100_F'] = lentil.fourier.dft2(np.ones((n, n)), 1 / n, shift=shift)
    d['shift100_shift'] = shift
    # sliced + offset == full (tests/test_fourier.py:81-94)
    f = np.zeros((10, 10), dtype=complex)
    f[4:7, 2:5] = crand(3, 3)
    slc = lentil.helper.boundary_slice(f)
    d['offset_f'] = f
    d['offset_slice'] = np.array([slc[0].start, slc[0].stop, slc[1].start, slc[1].stop])
    d['offset_offset'] = np.asarray(lentil.helper.slice_offset(slc, f.shape))
    d['offset_F'] = lentil.fourier.dft2(f, alpha=1 / 3, shape=10)
    # idft2
    for name, n in (('ieven', 10), ('iodd', 11)):
        F = crand(n, n)
        d[f'{name}_F'] = F
        d[f'{name}_f'] = lentil.fourier.idft2(F, 1 / n, unitary=False)
    d['names'] = np.array(names)
    np.savez_compressed(os.path.join(HERE, 'dft2.npz'), **d)

    # ---------------------------------------------------------- propagate
    p = {}

    def pupil(shape, radius, coeffs, focal_length=10, diameter=1, antialias=True):
        amp = lentil.normalize_power(lentil.circle(shape, radius, antialias=antialias))
        opd = lentil.zernike_compose(amp, coeffs) if coeffs is not None else 0
        return lentil.Pupil(amplitude=amp, opd=opd, pixelscale=diameter / (2 * radius),
                            focal_length=focal_length), amp, opd

    def run(name, pl, amp, opd, mask3d=None, wl=650e-9, fit_tilt=False, **kw):
        # fit_tilt may modify the OPD array in place: keep the input as given
        opd = np.array(np.broadcast_to(np.asarray(pl.opd, float), np.shape(amp)), copy=True)
        if fit_tilt:
            pl.fit_tilt(inplace=True)
        w = lentil.Wavefront(wl) * pl
        w = lentil.propagate_dft(w, **kw)
        p[f'{name}_amp'] = np.asarray(amp, float)
        p[f'{name}_opd'] = opd
        if mask3d is not None:
            p[f'{name}_mask'] = np.asarray(mask3d, float)
        p[f'{name}_pixelscale_in'] = np.asarray(pl.pixelscale, float)
        p[f'{name}_focal_length'] = np.asarray(pl.focal_length, float)
        p[f'{name}_wavelength'] = np.asarray(wl, float)
        p[f'{name}_fit_tilt'] = np.asarray(fit_tilt)
        for k in ('pixelscale', 'shape', 'prop_shape', 'oversample'):
            v = kw.get(k)
            p[f'{name}_{k}'] = np.asarray(-1 if v is None else v)
        if 'mask' in kw:
            p[f'{name}_outmask'] = np.asarray(kw['mask'], float)
        p[f'{name}_intensity'] = w.intensity
        p[f'{name}_nfields'] = np.asarray(len(w.data))
        return w

    # config-1 workload: 256^2 circle (non-antialiased), Noll 2-11 ~ N(0, 20 nm)
    c = np.concatenate([[0.0], rng.normal(0, 20e-9, 10)])
    amp = lentil.normalize_power(lentil.circle((256, 256), 128, antialias=False))
    opd = lentil.zernike_compose(amp, c)
    pl = lentil.Pupil(amplitude=amp, opd=opd, pixelscale=1 / 256, focal_length=10)
    run('config1', pl, amp, opd, pixelscale=5e-6, shape=128, oversample=2)

    # tilt with and without fit_tilt (tests/test_propagate.py:45-131)
    coeffs = [0, 2.1e-6, -1.3e-6]
    for ft in (False, True):
        pl, amp, opd = pupil((128, 128), 60, coeffs)
        run(f'tilt_fit{int(ft)}', pl, amp, opd, fit_tilt=ft, pixelscale=5e-6,
            shape=48, oversample=3)
    # output mask (tests/test_propagate_mask.py)
    pl, amp, opd = pupil((128, 128), 60, [0, 1e-7, 2e-7, 5e-8])
    mask = lentil.rectangle((128, 128), 48, 40, shift=(10, -15), antialias=False)
    run('outmask', pl, amp, opd, pixelscale=5e-6, shape=64, oversample=2, mask=mask)
    # everything tilted out of the window (tests/test_propagate.py:134-141)
    pl, amp, opd = pupil((127, 127), 60, [0, 1e-3])
    run('nooutput', pl, amp, opd, fit_tilt=True, pixelscale=5e-6, shape=32, oversample=2)
    # prop_shape < shape, odd shapes, rectangular output
    pl, amp, opd = pupil((101, 99), 45, [0, 3e-7, -2e-7, 1e-7, 4e-8])
    run('oddrect', pl, amp, opd, pixelscale=4e-6, shape=(45, 37), prop_shape=(21, 17),
        oversample=3)
    # segmented aperture: 3-D mask, per-segment fields, with and without fit_tilt
    segs = lentil.hex_segments(rings=1, seg_radius=14, seg_gap=2)
    H = segs.shape[1]
    gmask = np.sum(segs, axis=0)
    amp = lentil.normalize_power(gmask)
    opd = np.zeros_like(amp)
    for k in range(segs.shape[0]):
        r, cc = lentil.helper.mesh(amp.shape)
        ptt = rng.normal(0, 50e-9, 3)
        opd += segs[k] * (ptt[0] + ptt[1] * r / H + ptt[2] * cc / H)
    for ft in (False, True):
        pl = lentil.Pupil(amplitude=amp, opd=opd, mask=segs, pixelscale=1 / H,
                          focal_length=10)
        run(f'seg_fit{int(ft)}', pl, amp, opd, mask3d=segs, fit_tilt=ft, wl=550e-9,
            pixelscale=20e-6, shape=40, oversample=2)
    # small broadband accumulation through Wavefront.insert
    pl, amp, opd = pupil((64, 64), 30, [0, 0, 0, 5e-8, 2e-8])
    wl = np.array([500e-9, 620e-9, 780e-9])
    wt = np.array([0.2, 0.5, 0.3])
    img = np.zeros((48, 48))
    for lam, w8 in zip(wl, wt):
        w = lentil.propagate_dft(lentil.Wavefront(lam) * pl, pixelscale=6e-6, shape=24,
                                 oversample=2)
        img = w.insert(img, weight=w8)
    p['bb_amp'], p['bb_opd'], p['bb_wl'], p['bb_wt'], p['bb_img'] = amp, opd, wl, wt, img
    p['bb_pixelscale_in'] = np.asarray(pl.pixelscale, float)
    np.savez_compressed(os.path.join(HERE, 'propagate.npz'), **p)

    # -------------------------------------------------------------- fields
    fd = {}
    a = lentil.field.Field(data=np.ones((5, 4)), pixelscale=1, offset=[-2, -2])
    b = lentil.field.Field(data=np.ones((3, 3)), pixelscale=1, offset=[0, -1])
    c = lentil.field.merge(a, b)
    fd['merge_data'], fd['merge_offset'] = c.data, np.asarray(c.offset)
    fs = [lentil.field.Field(data=crand(5, 6), pixelscale=1, offset=[0, 0]),
          lentil.field.Field(data=crand(4, 4), pixelscale=1, offset=[2, 3]),
          lentil.field.Field(data=crand(3, 3), pixelscale=1, offset=[20, 20]),
          lentil.field.Field(data=crand(7, 2), pixelscale=1, offset=[-3, -4])]
    for k, f in enumerate(fs):
        fd[f'reduce_in{k}_data'], fd[f'reduce_in{k}_offset'] = f.data, np.asarray(f.offset)
    red = lentil.field.reduce(fs)
    fd['reduce_n'] = np.asarray(len(red))
    for k, f in enumerate(red):
        fd[f'reduce_out{k}_data'], fd[f'reduce_out{k}_offset'] = f.data, np.asarray(f.offset)
    out = np.zeros((9, 8))
    for f in fs:
        out = lentil.field.insert(f, out, intensity=True, weight=0.7)
    fd['insert_intensity'] = out
    out = np.zeros((9, 8), dtype=complex)
    for f in fs:
        out = lentil.field.insert(f, out)
    fd['insert_complex'] = out
    np.savez_compressed(os.path.join(HERE, 'field.npz'), **fd)

    # ------------------------------------------------------------ detector
    dd = {}
    for name, n, os_ in (('px64os2', 64, 2), ('px90os3', 90, 3), ('px128os4', 128, 4)):
        img = rng.uniform(0, 1, (n, n)) ** 4
        dd[f'{name}_img'] = img
        dd[f'{name}_os'] = np.asarray(os_)
        dd[f'{name}_pixel'] = lentil.detector.pixel(img, os_)
        dd[f'{name}_pixelate'] = lentil.detector.pixelate(img, os_)
    # sizes that are not a multiple of oversample: off-grid spline resampling
    # (own generator, so the cases above keep their inputs)
    rng_off = np.random.default_rng(20261204)
    for name, n, os_ in (('px100os3', 100, 3), ('px75os2', 75, 2), ('px61os7', 61, 7),
                         ('px128os3', 128, 3), ('px64os5', 64, 5)):
        img = rng_off.uniform(0, 1, (n, n)) ** 4
        dd[f'{name}_img'] = img
        dd[f'{name}_os'] = np.asarray(os_)
        dd[f'{name}_pixel'] = lentil.detector.pixel(img, os_)
        dd[f'{name}_pixelate'] = lentil.detector.pixelate(img, os_)
    np.savez_compressed(os.path.join(HERE, 'detector.npz'), **dd)

    # ---------------------------------------------------------- generators
    g = {}
    g['circle'] = lentil.circle((64, 70), 20.3, shift=(1.5, -2.25))
    g['circle_noaa'] = lentil.circle((64, 64), 20, antialias=False)
    g['hexagon'] = lentil.hexagon((64, 64), 20, shift=(2, -3))
    g['hexagon_rot'] = lentil.hexagon((64, 64), 20, rotate=True)
    g['rectangle'] = lentil.rectangle((64, 64), 30, 12, shift=(3, 4), angle=30)
    g['spider'] = lentil.spider((64, 64), 3, angle=210)
    g['hexseg'] = lentil.hex_segments(rings=2, seg_radius=10, seg_gap=1)
    m = lentil.circle((64, 64), 30)
    g['zcoeffs'] = rng.normal(0, 1e-7, 22)
    g['zcompose'] = lentil.zernike_compose(m, g['zcoeffs'])
    mm = g['hexseg'][4]
    rho, theta = lentil.zernike_coordinates(mm)
    g['zcoord_rho'], g['zcoord_theta'] = rho, theta
    g['zcompose_seg'] = lentil.zernike_compose(mm, [1e-8, 2e-8, -3e-8], rho=rho, theta=theta)
    g['psd'] = lentil.power_spectrum(m, 1 / 64, 25e-9, 8, 2, seed=7)
    wl = np.linspace(500, 900, 64)
    bb = lentil.radiometry.Blackbody(wl, 5800).value
    g['bb_wl_nm'], g['bb_value'] = wl, bb
    np.savez_compressed(os.path.join(HERE, 'generators.npz'), **g)

    # ------------------------------------------------------- propagate_fft
    # own generator so that the fixtures above do not change
    rf = np.random.default_rng(20261204)
    q = {}

    def fft_case(name, pl, wl, keep=48, **kw):
        w = lentil.propagate_fft(lentil.Wavefront(wl) * pl, **kw)
        field = w.data[0].data
        q[f'{name}_amp'] = np.asarray(pl.amplitude, float)
        q[f'{name}_opd'] = np.array(np.broadcast_to(np.asarray(pl.opd, float), pl.amplitude.shape))
        q[f'{name}_pixelscale_in'] = np.asarray(pl.pixelscale, float)
        q[f'{name}_focal_length'] = np.asarray(pl.focal_length, float)
        q[f'{name}_wavelength'] = np.asarray(wl, float)
        q[f'{name}_pixelscale'] = np.asarray(kw['pixelscale'], float)
        q[f'{name}_shape'] = np.asarray(-1 if kw.get('shape') is None else kw['shape'])
        q[f'{name}_oversample'] = np.asarray(kw.get('oversample', 2))
        q[f'{name}_scratch'] = np.asarray(-1 if kw.get('scratch') is None else kw['scratch'].shape)
        q[f'{name}_intensity'] = w.intensity
        q[f'{name}_out_shape'] = np.asarray(w.shape)
        q[f'{name}_out_wavelength'] = np.asarray(w.wavelength, float)
        q[f'{name}_out_pixelscale'] = np.asarray(w.pixelscale, float)
        q[f'{name}_field_shape'] = np.asarray(field.shape)
        # centre crop of the full FFT field (the whole array is large)
        k = min(keep, *field.shape)
        r0, c0 = (field.shape[0] - k) // 2, (field.shape[1] - k) // 2
        q[f'{name}_field_crop'] = field[r0:r0 + k, c0:c0 + k]
        q[f'{name}_field_crop_origin'] = np.asarray([r0, c0])
        if kw.get('scratch') is not None:     # lentil leaves the padded field in scratch
            reg = kw['scratch'][:field.shape[0], :field.shape[1]]
            q[f'{name}_scratch_sum'] = np.asarray(reg.sum())
            q[f'{name}_scratch_crop'] = reg[r0:r0 + k, c0:c0 + k]

    # the monochromatic workload pupil: fft shape 666 (even), cropped to 256^2
    c = np.concatenate([[0.0], rf.normal(0, 20e-9, 10)])
    amp = lentil.normalize_power(lentil.circle((256, 256), 128, antialias=False))
    pl = lentil.Pupil(amplitude=amp, opd=lentil.zernike_compose(amp, c), pixelscale=1 / 256,
                      focal_length=10)
    fft_case('c1', pl, 650e-9, pixelscale=5e-6, shape=128, oversample=2)
    # odd pupil, per-axis pixelscale, odd fft shape (153 x 191), shape=None, oversample 1
    amp = lentil.normalize_power(lentil.circle((127, 127), 60))
    opd = lentil.zernike_compose(amp, np.concatenate([[0.0], rf.normal(0, 40e-9, 8)]))
    pl = lentil.Pupil(amplitude=amp, opd=opd, pixelscale=1 / 127, focal_length=10)
    lam = (1 / 127) * 5e-6 * 153 / 10
    fft_case('odd', pl, lam, pixelscale=(5e-6, 4e-6), oversample=1)
    # the same through a scratch array (lentil centres by field.insert there)
    scratch = np.full((160, 200), 7 + 0j)
    fft_case('odd_scratch', pl, lam, pixelscale=(5e-6, 4e-6), oversample=1, scratch=scratch)
    # field larger than the fft shape: lentil's pad crops it (fft 151 x 151)
    amp = lentil.normalize_power(lentil.circle((200, 200), 98))
    opd = lentil.zernike_compose(amp, np.concatenate([[0.0], rf.normal(0, 30e-9, 6)]))
    pl = lentil.Pupil(amplitude=amp, opd=opd, pixelscale=1 / 200, focal_length=10)
    fft_case('crop', pl, (1 / 200) * 5e-6 * 151 / 10, pixelscale=5e-6, shape=(60, 70),
             oversample=1)
    # scratch_shape over a wavelength list
    q['scratch_shape_args'] = np.asarray([1 / 256, 5e-6, 10, 2])
    q['scratch_shape_wl'] = np.asarray([500e-9, 650e-9, 900e-9])
    q['scratch_shape'] = np.asarray(lentil.scratch_shape([500e-9, 650e-9, 900e-9], 1 / 256,
                                                         5e-6, 10, 2))
    np.savez_compressed(os.path.join(HERE, 'propagate_fft.npz'), **q)

    # ------------------------------------------- tilt planes (grism, Tilt)
    # own generator so that the fixtures above do not change
    rt = np.random.default_rng(20261205)
    t = {}
    # name: (trace, dispersion); meters on the focal plane, meters of
    # wavelength.  lentil 0.8.8 cannot evaluate a trace of order > 1 under
    # numpy 2 (leastsq hands scipy's quad a 1-element array: TypeError), so
    # the fixtures hold first-order traces only; a dispersion of order > 1
    # evaluates (__shift__ below) but its 1-element shift then fails in
    # propagate_dft's window arithmetic, so the images use first-order grisms
    grisms = {
        'lin': ([0.3, 0.0], [1e-3, 650e-9]),
        'steep': ([-2.5, 0.0], [8e-4, 600e-9]),
        'quad_disp': ([0.3, 0.0], [2.0, 1e-3, 650e-9]),
        'cubic_disp': ([0.0, 0.0], [-50.0, 1.5, 1.2e-3, 640e-9]),
    }
    wl = np.linspace(550e-9, 750e-9, 9)
    starts = np.array([[0.0, 0.0], [1e-6, -2e-6]])
    for name, (trace, disp) in grisms.items():
        dt = lentil.DispersiveTilt(trace=trace, dispersion=disp)
        xy = np.empty((len(starts), len(wl), 2))
        for i, (xs, ys) in enumerate(starts):
            for j, lam in enumerate(wl):
                x, y = dt.__shift__(wavelength=lam, xs=xs, ys=ys)
                xy[i, j] = float(np.squeeze(x)), float(np.squeeze(y))
        t[f'{name}_trace'] = np.asarray(trace, float)
        t[f'{name}_dispersion'] = np.asarray(disp, float)
        t[f'{name}_xy'] = xy
    t['wl'], t['starts'] = wl, starts
    # dispersed broadband images through lentil's loop, and a plain Tilt plane
    amp = lentil.normalize_power(lentil.circle((64, 64), 30))
    opd = lentil.zernike_compose(amp, np.concatenate([[0.0], rt.normal(0, 30e-9, 6)]))
    pl = lentil.Pupil(amplitude=amp, opd=opd, pixelscale=1 / 60, focal_length=10)
    t['img_amp'], t['img_opd'] = amp, opd
    t['img_wl'] = np.linspace(600e-9, 700e-9, 5)
    t['img_wt'] = rt.uniform(0.5, 1.0, 5)
    planes = {'lin': lentil.DispersiveTilt(trace=grisms['lin'][0], dispersion=grisms['lin'][1]),
              'steep': lentil.DispersiveTilt(trace=grisms['steep'][0],
                                             dispersion=grisms['steep'][1]),
              'tilt': lentil.Tilt(x=2.3e-6, y=-1.1e-6)}
    for name, tp in planes.items():
        img = np.zeros((96, 96))
        for lam, w8 in zip(t['img_wl'], t['img_wt']):
            w = lentil.propagate_dft(lentil.Wavefront(lam) * pl * tp, pixelscale=6e-6, shape=48,
                                     oversample=2)
            img = w.insert(img, weight=w8)
        t[f'img_{name}'] = img
    np.savez_compressed(os.path.join(HERE, 'tilt.npz'), **t)
    print('golden fixtures written to', HERE)


if __name__ == '__main__':
    if len(sys.argv) != 2 or not os.path.isfile(os.path.join(sys.argv[1], 'lentil', '__init__.py')):
        sys.exit('usage: make_golden.py <lentil-source-root>  (the directory holding lentil/)')
    main(sys.argv[1])
