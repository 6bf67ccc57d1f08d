"""Writes tests/golden/reference_kats.json: the known-answer cases that the
reference crate's own unit tests assert (bhtsne 0.7.10), restated as data.

The reference is Rust and cannot be built or run in this environment (no
cargo/rustc on either machine), so its outputs cannot be captured directly;
these cases are the values and tolerances its tests check, with the test that
holds each. tests/test_oracle.py pins the CPU oracle against them, and the GPU
tests compare the CUDA library with that pinned oracle.

Run: python tests/golden/make_golden.py
"""
import json
import math
import os

HERE = os.path.dirname(os.path.abspath(__file__))


def main():
    two32 = 2 ** 32
    kats = {
        "source": "bhtsne 0.7.10 unit tests (Rust), restated as data",
        "morton2_known_z_order": {
            "cite": "src/tsne/morton/d2.rs:69-75",
            "cases": [[[0, 0], 0], [[1, 0], 1], [[0, 1], 2], [[1, 1], 3]],
        },
        "morton2_sorting_groups_quadrants": {
            "cite": "src/tsne/morton/d2.rs:79-94",
            "ascending": [[1, 1], [5, 7], [2 ** 31, 2 ** 31]],
        },
        "morton3_known_z_order": {
            "cite": "src/tsne/morton/d3.rs:72-79",
            "cases": [[[0, 0, 0], 0], [[1, 0, 0], 1], [[0, 1, 0], 2], [[0, 0, 1], 4], [[1, 1, 1], 7]],
        },
        "quantize_spans_bucket_range": {
            "cite": "src/tsne/morton/d2.rs:98-115",
            "min": [0.0, -2.0],
            "extent": [4.0, 8.0],
            "scale": two32,
            "max_bucket": two32 - 1,
            "low": {"point": [0.0, -2.0], "expect": [0, 0]},
            "high": {"point": [4.0, 6.0], "expect": [two32 - 1, two32 - 1]},
            "mid": {"point": [2.0, 2.0], "expect": "strictly inside (0, max_bucket)"},
        },
        "quantize_zero_width_axis": {
            "cite": "src/tsne/morton/d2.rs:118-126",
            "min": [1.0, 5.0],
            "inv_scale": [0.0, two32 / 4.0],
            "point": [1.0, 7.0],
            "expect_axis0": 0,
            "expect_axis1_positive": True,
        },
        "search_beta_below_one": {
            "cite": "src/test.rs:1024-1049",
            "distances": [math.sqrt(20.0 + 100.0 * (i + 1.0) / 90.0) for i in range(90)],
            "perplexity": 30.0,
            "dtype": "f64",
            "effective_perplexity_tolerance": 0.1,
        },
        "fft_round_trip_2d": {"cite": "src/tsne/fft.rs:255-274", "m": 12, "tolerance": 1e-12},
        "fft_round_trip_1d": {"cite": "src/tsne/fft.rs:276-291", "m": 16, "tolerance": 1e-12},
        "fft_circular_convolution_2d": {"cite": "src/tsne/fft.rs:293-333", "m": 8, "tolerance": 1e-10},
        "lagrange_partition_of_unity": {"cite": "src/tsne/interpolation.rs:583-606", "steps": 11,
                                        "tolerance": 1e-12},
        "interpolation_vs_brute_force_2d": {"cite": "src/tsne/interpolation.rs:520-553", "n": 800,
                                            "uniform": [-5.0, 5.0], "z_rel": 1e-3, "force_rel_l2": 3e-2},
        "interpolation_vs_brute_force_1d": {"cite": "src/tsne/interpolation.rs:556-581", "n": 500,
                                            "uniform": [-4.0, 4.0], "z_rel": 1e-3, "force_rel_l2": 3e-2},
        "arena_conserves_points_2d": {"cite": "src/tsne/arena.rs:507-517", "n": 2000, "lcg_seed": 17,
                                      "offset": 100.0},
        "arena_conserves_points_3d": {"cite": "src/tsne/arena.rs:519-525", "n": 1500, "lcg_seed": 23},
        "arena_root_com_is_mean": {"cite": "src/tsne/arena.rs:527-537", "n": 1000, "lcg_seed": 5,
                                   "tolerance": 1e-3},
        "arena_duplicates_collapse": {"cite": "src/tsne/arena.rs:539-551", "n": 500, "value": 3.5,
                                      "expect_nodes": 1},
        "arena_single_point": {"cite": "src/tsne/arena.rs:553-561", "point": [2.0, -1.0]},
        "arena_coms_within_cells": {"cite": "src/test.rs:1165-1176, src/tsne/arena.rs:432-463",
                                    "n": 2000, "lcg_seed": 17, "offset": 100.0, "slack_fraction": 0.03},
        "learning_rate": {
            "cite": "src/test.rs:26-69",
            "cases": [[100, 12.0, 50.0], [120000, 12.0, 120000.0 / 12.0 / 4.0]],
            "n10000_range": [205.0, 212.0],
            "halving_exaggeration_doubles": [120000, 6.0],
        },
        "clusters_separate_large_scale": {"cite": "src/test.rs:1055-1120", "n_per_cluster": 150, "dim": 10,
                                          "centres": [0.0, 30.0], "noise_scale": 6.0, "lcg_seed": 42,
                                          "perplexity": 30.0, "epochs": 500, "theta": 0.5, "min_fraction": 0.95},
        "no_collapse": {"cite": "src/test.rs:1189-1224", "n": 500, "dim": 8, "lcg_seed": 23, "perplexity": 30.0,
                        "epochs": 1000, "theta": 0.5, "min_distinct_fraction": 0.5},
        "kl_finite_nonnegative": {"cite": "src/test.rs:148-205", "n": 60, "dim": 4, "lcg_seed": 7,
                                  "perplexity": 10.0, "epochs": 100},
        "with_neighbors_equals_metric_path": {"cite": "src/test.rs:888-928", "n": 80, "dim": 4, "lcg_seed": 11,
                                              "seed_lcg": 99, "perplexity": 10.0, "epochs": 100, "theta": 0.5},
    }
    with open(os.path.join(HERE, "reference_kats.json"), "w") as f:
        json.dump(kats, f, indent=1)
        f.write("\n")


if __name__ == "__main__":
    main()
