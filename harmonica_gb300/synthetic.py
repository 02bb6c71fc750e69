"""
Seeded synthetic prism layers and surveys with the sizes of the standard
benchmark workloads (no public dataset is involved; these stand in for the
ETOPO-based layers of harmonica's gallery, doc/gallery_src/forward/).

* ``layer_topography_1e4`` : 100 x 100 prisms on a 1 km grid over
  [0, 100 km]^2, bottoms at -30 000 m, tops a sum of 20 Gaussians (centres
  uniform in the region, amplitudes N(0, 800 m), widths U(5, 30) km, seed 0),
  densities U(2000, 3000) kg/m^3 (seed 1); 50 x 50 stations at 1000 m.
* ``layer_topography_1e6`` : 1000 x 1000 prisms on a 200 m grid (200 km
  square), bottoms at -10 000 m, Gaussian-sum tops (seed 2), densities
  U(1800, 3100) (seed 2); 500 x 500 stations at 2000 m + N(0, 50 m) (seed 3).
* ``batched_problems`` : 256 uneven independent problems (g_z / g_zz).
* ``serving_stream`` : a Poisson stream of forward-solve requests.
"""

import numpy as np


def gaussian_topography(easting, northing, region, n_bumps, seed):
    rng = np.random.default_rng(seed)
    w, e, s, n = region
    ce = rng.uniform(w, e, n_bumps)
    cn = rng.uniform(s, n, n_bumps)
    amp = rng.normal(0.0, 800.0, n_bumps)
    width = rng.uniform(5e3, 30e3, n_bumps)
    ge, gn = np.meshgrid(easting, northing)
    top = np.zeros_like(ge)
    for k in range(n_bumps):
        top += amp[k] * np.exp(-((ge - ce[k]) ** 2 + (gn - cn[k]) ** 2) / (2 * width[k] ** 2))
    return top


def layer_topography_1e4():
    """Returns dict(easting, northing, top, bottom, density, coordinates)."""
    spacing = 1000.0
    easting = np.arange(100) * spacing + spacing / 2
    northing = np.arange(100) * spacing + spacing / 2
    region = (0.0, 100e3, 0.0, 100e3)
    top = gaussian_topography(easting, northing, region, 20, seed=0)
    bottom = np.full_like(top, -30000.0)
    density = np.random.default_rng(1).uniform(2000, 3000, top.shape)
    se, sn = np.meshgrid(np.linspace(0, 100e3, 50), np.linspace(0, 100e3, 50))
    coordinates = (se.ravel(), sn.ravel(), np.full(se.size, 1000.0))
    return dict(easting=easting, northing=northing, top=top, bottom=bottom, density=density,
                coordinates=coordinates)


def layer_topography_1e6(n_side=1000, n_stations_side=500):
    """The 1e6-prism layer (or a smaller one with the same recipe)."""
    spacing = 200e3 / n_side
    easting = np.arange(n_side) * spacing + spacing / 2
    northing = np.arange(n_side) * spacing + spacing / 2
    region = (0.0, 200e3, 0.0, 200e3)
    top = gaussian_topography(easting, northing, region, 20, seed=2)
    bottom = np.full_like(top, -10000.0)
    density = np.random.default_rng(2).uniform(1800, 3100, top.shape)
    se, sn = np.meshgrid(
        np.linspace(0, 200e3, n_stations_side), np.linspace(0, 200e3, n_stations_side)
    )
    up = 2000.0 + np.random.default_rng(3).normal(0.0, 50.0, se.size)
    coordinates = (se.ravel(), sn.ravel(), up)
    return dict(easting=easting, northing=northing, top=top, bottom=bottom, density=density,
                coordinates=coordinates)


def layer_to_prisms(layer):
    """(M, 6) prism array and (M,) densities of a layer dict, row-major (northing, easting)."""
    e, n = layer["easting"], layer["northing"]
    he, hn = (e[1] - e[0]) / 2, (n[1] - n[0]) / 2
    ge, gn = np.meshgrid(e, n)
    prisms = np.column_stack(
        [ge.ravel() - he, ge.ravel() + he, gn.ravel() - hn, gn.ravel() + hn,
         layer["bottom"].ravel(), layer["top"].ravel()]
    )
    return prisms, layer["density"].ravel()


def batched_problems(n_problems=256, seed=4, scale=1.0):
    """
    The batched workload: ``n_problems`` independent problems with prism
    counts log-uniform in [1e3, 2e5] and station counts log-uniform in
    [1e3, 5e4] (both times ``scale``), random axis-aligned prisms with sides
    U(50, 2000) m in a 50 km square, tops U(-5000, 1000) m and bottoms
    top - U(50, 2000) m, densities U(-500, 500), stations uniform in the
    prisms' bounding box at heights U(100, 3000) m; fields alternate g_z and
    g_zz.  Returns a list of dicts (coordinates, prisms, density, field).
    """
    rng = np.random.default_rng(seed)
    problems = []
    for p in range(n_problems):
        m = max(1, int(round(np.exp(rng.uniform(np.log(1e3), np.log(2e5))) * scale)))
        n = max(1, int(round(np.exp(rng.uniform(np.log(1e3), np.log(5e4))) * scale)))
        west = rng.uniform(0, 50e3, m)
        south = rng.uniform(0, 50e3, m)
        top = rng.uniform(-5000, 1000, m)
        prisms = np.column_stack(
            [west, west + rng.uniform(50, 2000, m), south, south + rng.uniform(50, 2000, m),
             top - rng.uniform(50, 2000, m), top]
        )
        density = rng.uniform(-500, 500, m)
        lo_e, hi_e = prisms[:, 0].min(), prisms[:, 1].max()
        lo_n, hi_n = prisms[:, 2].min(), prisms[:, 3].max()
        coordinates = (rng.uniform(lo_e, hi_e, n), rng.uniform(lo_n, hi_n, n),
                       rng.uniform(100, 3000, n))
        problems.append(dict(coordinates=coordinates, prisms=prisms, density=density,
                             field="g_z" if p % 2 == 0 else "g_zz"))
    return problems


def basement_layer(n_side=200, spacing=500.0, seed=5, noise_seed=6, n_stations_side=100,
                   height=500.0, contrast=-400.0):
    """
    The basement-inversion workload: an n_side x n_side layer of 500 m cells
    (100 km square) with tops at 0 m and bottoms a smooth seeded surface
    (Gaussian-filtered white noise rescaled to mean -3000 m, std 800 m), a
    density contrast of -400 kg/m^3, and g_z data on an n x n station grid at
    ``height`` computed elsewhere; returns the geometry and the true bottom.
    """
    rng = np.random.default_rng(seed)
    noise = rng.normal(size=(n_side, n_side))
    k = np.fft.fftfreq(n_side)
    kx, ky = np.meshgrid(k, k)
    sigma = 5.0  # cells
    filt = np.exp(-2 * (np.pi * sigma) ** 2 * (kx ** 2 + ky ** 2))
    smooth = np.real(np.fft.ifft2(np.fft.fft2(noise) * filt))
    smooth = (smooth - smooth.mean()) / smooth.std()
    bottom = -3000.0 + 800.0 * smooth
    bottom = np.minimum(bottom, -10.0)  # keep bottom below the 0 m top
    easting = np.arange(n_side) * spacing + spacing / 2
    northing = np.arange(n_side) * spacing + spacing / 2
    side = n_side * spacing
    se, sn = np.meshgrid(np.linspace(0, side, n_stations_side),
                         np.linspace(0, side, n_stations_side))
    coordinates = (se.ravel(), sn.ravel(), np.full(se.size, height))
    return dict(easting=easting, northing=northing, top=np.zeros_like(bottom), bottom=bottom,
                density=np.full_like(bottom, contrast), coordinates=coordinates,
                noise_seed=noise_seed)


# WGS84 semi-axes (metres)
_WGS84_A = 6378137.0
_WGS84_B = 6356752.314245179


def geocentric_radius(latitude):
    """Geocentric radius of the WGS84 ellipsoid at geodetic latitudes (degrees)."""
    phi = np.radians(latitude)
    a, b = _WGS84_A, _WGS84_B
    num = (a**2 * np.cos(phi)) ** 2 + (b**2 * np.sin(phi)) ** 2
    den = (a * np.cos(phi)) ** 2 + (b * np.sin(phi)) ** 2
    return np.sqrt(num / den)


def tesseroid_layer_andes(spacing=0.1, station_spacing=0.5, height=10e3, seed=9):
    """
    Tesseroid layer with the shape of harmonica's tesseroid-layer gallery
    example (doc/gallery_src/forward/tesseroid_layer.py): region
    (-78, -53, -57, -20) degrees on a 0.1-degree grid (251 x 371 =
    93,121 tesseroids), reference surface the WGS84 geocentric radius, density
    2670 kg/m^3 above it and 1040 - 2670 below, computation points on a
    0.5-degree grid (51 x 75 = 3,825) 10 km above the reference.  The
    topography is synthetic (seeded): a mountain range along -69 degrees
    (up to ~6 km) over an ocean floor of ~-4.5 km in the east and west,
    plus 40 random bumps.  Returns dict(tesseroids (M, 6), density (M,),
    coordinates (3 arrays), shape).
    """
    w, e, s, n = -78.0, -53.0, -57.0, -20.0
    lon = np.round(np.arange(w, e + spacing / 2, spacing), 10)
    lat = np.round(np.arange(s, n + spacing / 2, spacing), 10)
    glon, glat = np.meshgrid(lon, lat)
    rng = np.random.default_rng(seed)
    topo = 5500.0 * np.exp(-((glon + 69.0) ** 2) / (2 * 1.5**2)) - 4500.0 * (
        1 - np.exp(-((glon + 66.0) ** 2) / (2 * 9.0**2)))
    for _ in range(40):
        clon, clat = rng.uniform(w, e), rng.uniform(s, n)
        topo += rng.normal(0, 900.0) * np.exp(
            -((glon - clon) ** 2 + (glat - clat) ** 2) / (2 * rng.uniform(0.3, 2.0) ** 2))
    reference = geocentric_radius(glat)
    surface = topo + reference
    top = np.maximum(surface, reference)
    bottom = np.minimum(surface, reference)
    density = np.where(topo > 0, 2670.0, 1040.0 - 2670.0)
    h = spacing / 2
    tess = np.stack([glon - h, glon + h, glat - h, glat + h, bottom, top], axis=-1).reshape(-1, 6)
    slon = np.arange(w, e + station_spacing / 2, station_spacing)
    slat = np.arange(s, n + station_spacing / 2, station_spacing)
    plon, plat = np.meshgrid(slon, slat)
    coords = (plon.ravel(), plat.ravel(), geocentric_radius(plat).ravel() + height)
    return dict(tesseroids=tess, density=density.ravel(), coordinates=coords, shape=glon.shape)


def serving_models(n_models=24, seed=7):
    """Prism models of the serving workload: ``n_models`` random layers of
    200 m x 200 m prisms with log-uniform 1e3-1e6 prisms each (tops
    U(-3000, 1000) m, thicknesses U(100, 5000) m, densities U(1800, 3100)),
    spread over a square of side sqrt(M) x 200 m.  Returns a list of
    (prisms (M, 6), density (M,), side)."""
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(np.log(1e3), np.log(1e6), n_models)).astype(int)
    models = []
    for k, m in enumerate(sizes):
        r = np.random.default_rng(100 + k)
        side = np.sqrt(m) * 200.0
        west = r.uniform(0, side, m)
        south = r.uniform(0, side, m)
        top = r.uniform(-3000, 1000, m)
        prisms = np.column_stack([west, west + 200.0, south, south + 200.0,
                                  top - r.uniform(100, 5000, m), top])
        models.append((prisms, r.uniform(1800, 3100, m), side))
    return models


def serving_stream(rate=200.0, seconds=5.0, n_models=24, n_resident=8, resident_share=0.3,
                   seed=7):
    """
    The serving workload: Poisson arrivals at ``rate`` requests/s for
    ``seconds``; each request is a survey of log-uniform 1e3-2.5e5 stations
    scattered over one model of :func:`serving_models` at heights
    U(100, 3000) m, with a field drawn from (g_z, potential, g_zz);
    ``resident_share`` of the requests use one of the first ``n_resident``
    models as a resident layer, the others send their prisms.  Returns a list
    of dicts (t, n_stations, resident, model, field, seed); the stations are
    drawn from ``seed`` by :func:`serving_request_coordinates`.
    """
    rng = np.random.default_rng(seed)
    fields = ("g_z", "potential", "g_zz")
    t, out = 0.0, []
    while True:
        t += rng.exponential(1.0 / rate)
        if t >= seconds:
            return out
        n_st = int(np.exp(rng.uniform(np.log(1e3), np.log(2.5e5))))
        resident = bool(rng.uniform() < resident_share)
        k = int(rng.integers(0, n_resident)) if resident else int(rng.integers(n_resident,
                                                                               n_models))
        out.append(dict(t=t, n_stations=n_st, resident=resident, model=k,
                        field=fields[int(rng.integers(0, 3))], seed=int(rng.integers(1 << 30))))


def serving_request_coordinates(request, side):
    """Stations of one request of :func:`serving_stream` over a model of side ``side``."""
    r = np.random.default_rng(request["seed"])
    n = request["n_stations"]
    return (r.uniform(0, side, n), r.uniform(0, side, n), r.uniform(100, 3000, n))
