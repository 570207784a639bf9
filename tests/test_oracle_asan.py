"""The CPU oracle (oracle/prt_oracle.c, test infrastructure) compiled with
AddressSanitizer and UndefinedBehaviorSanitizer and driven over edge-case scenes: no
triangles, one, two, three, identical triangles, non-finite vertices, a random soup;
rays with zero direction components and non-finite values; every entry point (build,
node export, nearest hits on several threads, hit statistics, camera, Lambert).  The
checker must itself be free of invalid accesses and undefined behaviour."""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT

DRIVER = r"""
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "prt_oracle.h"

static unsigned long long st = 12345;
static float rnd(void) { /* splitmix-style, in [-1, 1) */
	st += 0x9E3779B97F4A7C15ull;
	unsigned long long z = st;
	z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
	z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
	z ^= z >> 31;
	return (float)((double)(z >> 40) / 8388608.0 - 1.0);
}

static void run(const float *tris, size_t n, const float *rays, size_t m) {
	orc_bvh *b = orc_bvh_build(tris, n);
	size_t nn = orc_bvh_node_count(b);
	orc_node *nodes = malloc((nn ? nn : 1) * sizeof *nodes);
	orc_bvh_nodes(b, nodes);
	orc_hit *hits = malloc((m ? m : 1) * sizeof *hits);
	orc_stats *stats = malloc((m ? m : 1) * sizeof *stats);
	orc_nearest_hits(b, rays, m, hits, 3);
	orc_hit_stats(b, rays, m, stats, 2);
	unsigned char *rgba = malloc(4 * (m ? m : 1));
	if (n)
		orc_lambert(tris, rays, hits, m, rgba);
	size_t valid = 0;
	for (size_t i = 0; i < m; ++i)
		valid += hits[i].valid;
	printf("%zu %zu %zu\n", n, nn, valid);
	free(rgba);
	free(stats);
	free(hits);
	free(nodes);
	orc_bvh_free(b);
}

int main(void) {
	enum { M = 3000, N = 2000 };
	float *rays = malloc(sizeof(float) * 6 * M);
	for (int i = 0; i < M; ++i)
		for (int k = 0; k < 6; ++k)
			rays[6 * i + k] = 3.0f * rnd();
	for (int i = 0; i < M; i += 7)
		rays[6 * i + 3 + i % 3] = 0.0f;             /* a zero direction component */
	rays[6 * 5 + 4] = NAN;
	rays[6 * 9 + 0] = INFINITY;
	float *tris = malloc(sizeof(float) * 9 * N);
	for (int i = 0; i < N; ++i) {
		float c[3] = {rnd(), rnd(), rnd()};
		for (int k = 0; k < 9; ++k)
			tris[9 * i + k] = c[k % 3] + 0.05f * rnd();
	}
	for (size_t n = 0; n <= 3; ++n)
		run(tris, n, rays, M);
	run(tris, N, rays, M);
	for (int i = 0; i < 64; ++i)                    /* identical triangles */
		memcpy(tris + 9 * i, tris, 9 * sizeof(float));
	tris[9 * 70 + 4] = NAN;                          /* non-finite vertices */
	tris[9 * 71 + 8] = -INFINITY;
	run(tris, N, rays, M);
	run(tris, N, rays, 0);
	orc_camera cam = {64, 48, 2, 0, {0.3f, 0.1f, -0.05f}, 0.05f, 0.05f, 0.0f,
	                  cosf(-1.58f), sinf(-1.58f)};
	float *crays = malloc(sizeof(float) * 6 * 64 * 48);
	for (unsigned f = 0; f < 3; ++f) {
		cam.form = f;
		cam.sensor_z = -0.25f;
		orc_camera_rays(&cam, crays);
		run(tris, N, crays, 64 * 48);
	}
	free(crays);
	free(tris);
	free(rays);
	return 0;
}
"""


def test_oracle_under_sanitizers(tmp_path):
    cc = shutil.which("gcc")
    if not cc:
        pytest.skip("no gcc")
    drv = tmp_path / "driver.c"
    drv.write_text(DRIVER)
    exe = tmp_path / "oracle_asan"
    cmd = [cc, "-std=c11", "-D_GNU_SOURCE", "-O1", "-g", "-ffp-contract=off",
           "-fsanitize=address,undefined", "-fno-sanitize-recover=undefined",
           f"-I{os.path.join(ROOT, 'oracle')}", os.path.join(ROOT, "oracle", "prt_oracle.c"),
           str(drv), "-o", str(exe), "-lpthread", "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0 and "asan" in r.stderr.lower():
        pytest.skip("AddressSanitizer runtime not available")
    assert r.returncode == 0, r.stderr
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=1")
    r = subprocess.run([str(exe)], capture_output=True, text=True, env=env, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    assert "runtime error" not in r.stderr and "AddressSanitizer" not in r.stderr, \
        r.stderr[-3000:]
    rows = [list(map(int, ln.split())) for ln in r.stdout.split("\n") if ln]
    assert len(rows) == 10
    assert [row[0] for row in rows[:4]] == [0, 1, 2, 3]
    assert rows[4][2] > 0  # the random soup is hit
