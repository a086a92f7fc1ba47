"""Known answers of the reference's own scale test, restated.

src/tests/scale/bench_select_scale.c:38-56 defines a closed-form table (id = i + 1,
region_id = i % 50, amount = i % 10000, needle_key = (i * 2654435761) mod 2^32) and :97-160 the
exact answers of its queries, checked by the cases at :1127-1170. These functions restate those
formulas; they pin the oracle and, on the GPU, the kernels directly.
"""

REGIONS = 50
AMOUNT_RANGE = 10000
HIGH_AMOUNT = 9990
ZONE_SIZE = 10
BIG_DIM_ROWS = 1000000
BIG_DIM_WEIGHTS = 100
KEY_MULTIPLIER = 2654435761


def sum_amount(n):  # ss_sum_amount :97-104
    full, rem = divmod(n, AMOUNT_RANGE)
    cycle = AMOUNT_RANGE * (AMOUNT_RANGE - 1) // 2
    return float(full * cycle + (rem * (rem - 1) // 2 if rem > 0 else 0))


def count_amount_above(n, threshold):  # ss_count_amount_above :106-114
    full, rem = divmod(n, AMOUNT_RANGE)
    per_cycle = AMOUNT_RANGE - 1 - threshold
    partial = rem - threshold - 1 if rem > threshold + 1 else 0
    return full * per_cycle + partial


def count_region(n, region):  # ss_count_region :116-120
    return n // REGIONS + (1 if n % REGIONS > region else 0)


def region_rows(n, region):  # ss_region_rows :123-127
    return n // REGIONS + (1 if n % REGIONS > region else 0)


def region_amount_sum(n, region):  # ss_region_amount_sum :129-138
    rows = region_rows(n, region)
    cycles, rem = divmod(rows, 200)
    cycle_sum = 200 * 199 // 2
    partial = rem * (rem - 1) // 2 if rem > 0 else 0
    return float(rows * region + 50 * (cycles * cycle_sum + partial))


def amount_rows(n, amount):  # ss_amount_rows :140-144
    return n // AMOUNT_RANGE + (1 if n % AMOUNT_RANGE > amount else 0)


def weight_sum(count):  # ss_weight_sum :147-154
    cycles, rem = divmod(count, BIG_DIM_WEIGHTS)
    partial = rem * (rem - 1) // 2 if rem > 0 else 0
    return float(cycles * (BIG_DIM_WEIGHTS * (BIG_DIM_WEIGHTS - 1) // 2) + partial)


def key_of_row(row):  # ss_key_of_row :156-160
    return (row * KEY_MULTIPLIER) & 0xFFFFFFFF


def key_is_searchable(key):  # ss_key_is_searchable :163-167
    return (1 << 24) <= key <= 0xFFFFFFFF - (1 << 24)


def needle_row(n):  # :1089-1094
    r = n // 2
    while not key_is_searchable(key_of_row(r)):
        r += 1
    return r


def id_range_count(n):  # "filter count, id range": id > 1000 AND id <= 900000000, :1141-1143
    return min(n, 900000000) - min(n, 1000)


def join_zone_expected(n, zone=2):  # :1112-1121, regions.zone = region_id / 10
    rows = sum(region_rows(n, r) for r in range(zone * ZONE_SIZE, (zone + 1) * ZONE_SIZE))
    amount = sum(region_amount_sum(n, r) for r in range(zone * ZONE_SIZE, (zone + 1) * ZONE_SIZE))
    return rows, amount


def expected(n):
    """The answers of the scale cases at n rows."""
    return {
        "sum_min_max_amount": [sum_amount(n), 0.0, float(min(AMOUNT_RANGE - 1, n - 1))],
        "count_amount_gt_9990": count_amount_above(n, HIGH_AMOUNT),
        "count_region_eq_7": count_region(n, 7),
        "count_id_range": id_range_count(n),
        "group_region": [[r, region_rows(n, r), region_amount_sum(n, r)] for r in range(REGIONS) if region_rows(n, r) > 0],
        "group_amount": [[a, amount_rows(n, a), amount_rows(n, a) * (a % REGIONS)] for a in range(AMOUNT_RANGE) if amount_rows(n, a) > 0],
        "join_zone2": list(join_zone_expected(n)),
        "needle_row": needle_row(n),
        "needle_key": key_of_row(needle_row(n)),
    }
