"""Icosahedral grid generator: topology, orientation and vertex placement."""
import numpy as np
import pytest

from conftest import ref_grid


def read_grid(path):
    lat, lon, fr, cent = [], [], [], []
    with open(path) as f:
        next(f)
        for line in f:
            a, b = line.split("{", 1)
            p = a.split()
            lat.append(float(p[1])); lon.append(float(p[2]))
            f_part, c_part = b.split("}", 1)
            fr.append([int(x) for x in f_part.split(",")])
            nums = c_part.replace("(", " ").replace(")", " ").replace(",", " ").replace("{", " ").replace("}", " ").split()
            cent.append([float(x) for x in nums])
    rc = np.pi / 180
    return np.array(lat) * rc, np.array(lon) * rc, np.array(fr), np.array(cent).reshape(-1, 6, 2) * rc


def xyz(lat, lon):
    return np.stack([np.cos(lat) * np.cos(lon), np.cos(lat) * np.sin(lon), np.sin(lat)], -1)


@pytest.mark.parametrize("level", [0, 1, 2, 3, 4, 5])
def test_counts_and_symmetry(grid_dir, level):
    lat, lon, fr, cent = read_grid(grid_dir / f"grid_{level}.txt")
    N = 10 * 4 ** level + 2
    assert len(lat) == N
    pent = fr[:, 5] < 0
    assert pent.sum() == 12
    for i in range(N):
        k = 5 if pent[i] else 6
        for j in range(k):
            f = fr[i, j]
            assert 0 <= f < N and f != i
            assert i in fr[f]                      # friendship is symmetric
    edges = (6 * (N - 12) + 60) // 2
    assert edges == 3 * N - 6


@pytest.mark.parametrize("level", [1, 3, 5])
def test_clockwise_and_circumcentres(grid_dir, level):
    lat, lon, fr, cent = read_grid(grid_dir / f"grid_{level}.txt")
    P = xyz(lat, lon)
    for i in range(0, len(lat), max(1, len(lat) // 400)):
        k = 5 if fr[i, 5] < 0 else 6
        for j in range(k):
            a, b = P[fr[i, j]], P[fr[i, (j + 1) % k]]
            # clockwise seen from outside: (a - p) x (b - p) points inwards
            assert np.dot(np.cross(a - P[i], b - P[i]), P[i]) < 0
            c = xyz(cent[i, j, 0], cent[i, j, 1])
            d = [np.arccos(np.clip(np.dot(c, q), -1, 1)) for q in (P[i], a, b)]
            assert max(d) - min(d) < 1e-12


@pytest.mark.parametrize("level", [2, 3, 4])
def test_same_layout_as_reference_files(grid_dir, level):
    """Generated and shipped grids agree in size, pentagon count and orientation convention."""
    lat, lon, fr, cent = read_grid(ref_grid(level))
    lat2, lon2, fr2, cent2 = read_grid(grid_dir / f"grid_{level}.txt")
    assert len(lat) == len(lat2)
    assert (fr[:, 5] < 0).sum() == (fr2[:, 5] < 0).sum() == 12
    P = xyz(lat, lon)
    i = 100
    k = 6 if fr[i, 5] >= 0 else 5
    assert np.dot(np.cross(P[fr[i, 0]] - P[i], P[fr[i, 1]] - P[i]), P[i]) < 0
    # cell sizes of the two grids have the same mean (equal-count grids on the unit sphere)
    def mean_spacing(lat, lon, fr):
        P = xyz(lat, lon)
        return np.mean([np.arccos(np.clip(np.dot(P[i], P[fr[i, 0]]), -1, 1)) for i in range(len(lat))])
    assert abs(mean_spacing(lat, lon, fr) / mean_spacing(lat2, lon2, fr2) - 1) < 0.05


def _parse_grid(path):
    """(node (lat, lon) strings, friends [N][6], centroids [N][6][2]) of a grid file."""
    import re
    names, fr, cen = [], [], []
    for line in open(path).read().splitlines()[1:]:
        a = line.split("{")
        head = a[0].split()
        names.append((head[1], head[2]))
        fr.append([int(x) for x in a[1].split("}")[0].split(",")])
        cen.append([(float(x), float(y)) for x, y in re.findall(r"\(([^,]+), ([^)]+)\)", a[2])])
    return names, np.array(fr), np.array(cen)


@pytest.mark.parametrize("level", [0, 2, 4, 5])
def test_oracle_generator_builds_the_same_mesh(grid_dir, tmp_path, level):
    """The oracle's own icosahedral generator (creation-order numbering) and the product's (depth-first
    numbering) describe the same mesh: identical node positions, friend cycles and circumcentres, bit for bit
    once the nodes are matched."""
    from oracle import pyoracle as O
    O.generate_grid_file(level, tmp_path / "o.txt")
    no, fo, co = _parse_grid(tmp_path / "o.txt")
    npn, fp, cp = _parse_grid(grid_dir / f"grid_{level}.txt")
    assert len(no) == len(npn) == 10 * 4 ** level + 2
    where = {n: i for i, n in enumerate(npn)}
    perm = np.array([where[n] for n in no])            # oracle node -> product node
    assert len(set(perm.tolist())) == len(no)
    mapped = np.where(fo >= 0, perm[np.maximum(fo, 0)], -1)
    np.testing.assert_array_equal(mapped, fp[perm])
    np.testing.assert_array_equal(co, cp[perm])


def test_oracle_loading_factors_match_product(built):
    import geodesicodis_gb300 as g
    from oracle import pyoracle as O
    a, b = O.loading_factors(0.113, 252.1e3, 32), g.loading_factors(0.113, 252.1e3, 32)
    np.testing.assert_array_equal(a[1:], b[1:])        # l = 0 is unused (the reference divides by l)
    np.testing.assert_array_equal(O.benchmark_sh_factors(0.113, 252.1e3, 16, 1),
                                  g.benchmark_sh_factors(0.113, 252.1e3, 16, 1))


def test_text_round16_is_printf_then_strtod(built):
    """odis_text_round16 (exact integer arithmetic, shared by the host and device generators) against
    float("%.16f" % v): Python's formatting and parsing round correctly, as glibc's printf and strtod do.
    Random values at every scale the generators meet, and values within a few ulps of a tie of the 16th
    decimal, where a one-ulp slip in the arithmetic would show."""
    import geodesicodis_gb300 as g
    rng = np.random.default_rng(2024)
    parts = [rng.uniform(-1, 1, 200000), rng.uniform(-360, 360, 50000),
             np.sign(rng.uniform(-1, 1, 100000)) * 10.0 ** rng.uniform(-25, 0, 100000),
             np.array([0.0, -0.0, 1.0, -1.0, 0.5, 1e-16, 5e-17, 4.9999999999999999e-17, 1.5e-16, 2.5e-16,
                       0.9999999999999999, 0.99999999999999995, 89.99999999999999, 1e-300, 5e-324])]
    k = rng.integers(0, 10 ** 16, 100000)
    ties = (k + 0.5) * 1e-16                                   # nearest doubles to ties of the 16th decimal
    parts += [ties, np.nextafter(ties, 0), np.nextafter(ties, 1), -ties]
    v = np.concatenate(parts)
    got = g.text_round16(v)
    want = np.array([float("%.16f" % x) for x in v])
    bad = np.flatnonzero(got.view(np.int64) != want.view(np.int64))
    assert bad.size == 0, [(v[i], got[i], want[i]) for i in bad[:5]]
