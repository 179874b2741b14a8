"""ctypes mirror of include/pilon_gb300.h.

These are the structs a JVM host would declare through JNI or the Java
foreign-function API; Python uses the same layout through ctypes.
"""
import ctypes as C

PG_OK = 0
PG_ERR_ARG = 1
PG_ERR_CUDA = 2
PG_ERR_NOMEM = 3
PG_ERR_INDEX = 4
PG_ERR_STATE = 5
PG_ERR_LIMIT = 6
PG_ERR_TIMEOUT = 7

STATUS_NAMES = {
    0: "PG_OK", 1: "PG_ERR_ARG", 2: "PG_ERR_CUDA", 3: "PG_ERR_NOMEM",
    4: "PG_ERR_INDEX", 5: "PG_ERR_STATE", 6: "PG_ERR_LIMIT", 7: "PG_ERR_TIMEOUT",
}

PG_NOT_LONG_READ, PG_NANOPORE, PG_PACBIO = 0, 1, 2
PG_BAM_FRAGS, PG_BAM_JUMPS, PG_BAM_UNPAIRED, PG_BAM_BAM = 0, 1, 2, 3

PG_CALL_HAS_BASE = 1 << 4
PG_CALL_HOMO = 1 << 5
PG_CALL_INS = 1 << 6
PG_CALL_DEL = 1 << 7
PG_CALL_HOMO_INDEL = 1 << 8
PG_CALL_CONFIRMED = 1 << 12
PG_CALL_DELETED = 1 << 13
PG_CHANGE_NONE, PG_CHANGE_SNP, PG_CHANGE_INS, PG_CHANGE_DEL, PG_CHANGE_AMB = 0, 1, 2, 3, 4


def call_base(f):
    return f & 3


def call_alt(f):
    return (f >> 2) & 3


def call_change(f):
    return (f >> 9) & 7


class pg_params(C.Structure):
    _fields_ = [
        ("min_mq", C.c_int32), ("min_qual", C.c_int32), ("flank", C.c_int32),
        ("default_qual", C.c_int32), ("min_min_depth", C.c_int32), ("nonpf", C.c_int32),
        ("duplicates", C.c_int32), ("old_indel", C.c_int32), ("fix_amb", C.c_int32),
        ("long_read", C.c_int32), ("bam_type", C.c_int32), ("long_read_only", C.c_int32),
        ("min_depth", C.c_double),
    ]


class pg_reads(C.Structure):
    _fields_ = [
        ("n_reads", C.c_int64),
        ("pos", C.c_void_p), ("aend", C.c_void_p), ("flag", C.c_void_p), ("mapq", C.c_void_p),
        ("tlen", C.c_void_p), ("ref_id", C.c_void_p), ("mate_ref_id", C.c_void_p),
        ("cigar_off", C.c_void_p), ("n_cigar", C.c_void_p), ("cigar", C.c_void_p),
        ("seq_off", C.c_void_p), ("l_seq", C.c_void_p), ("seq", C.c_void_p),
        ("qual_off", C.c_void_p), ("qual", C.c_void_p),
        ("n_cigar_words", C.c_int64), ("seq_bytes", C.c_int64), ("qual_bytes", C.c_int64),
    ]


class pg_region(C.Structure):
    _fields_ = [
        ("contig", C.c_int32), ("start", C.c_int32), ("stop", C.c_int32), ("pad_", C.c_int32),
        ("read_begin", C.c_int64), ("read_end", C.c_int64),
    ]


class pg_region_stats(C.Structure):
    _fields_ = [
        ("base_count", C.c_int64), ("read_count", C.c_int64),
        ("phys_cov_start", C.c_int32), ("insert_size_start", C.c_int32),
        ("min_depth", C.c_int32), ("n_changes", C.c_int32),
        ("fr_count", C.c_int64), ("fr_sum", C.c_int64), ("fr_sumsq", C.c_int64),
        ("rf_count", C.c_int64), ("rf_sum", C.c_int64), ("rf_sumsq", C.c_int64),
        ("error", C.c_int32), ("n_ins_strings", C.c_int32),
    ]


class pg_region_out(C.Structure):
    _fields_ = [
        ("count", C.c_void_p), ("qual_sum", C.c_void_p),
        ("mq_sum", C.c_void_p), ("q_sum", C.c_void_p), ("phys_cov", C.c_void_p),
        ("insert_size", C.c_void_p), ("bad_pair", C.c_void_p),
        ("deletions", C.c_void_p), ("del_qual", C.c_void_p), ("insertions", C.c_void_p),
        ("ins_qual", C.c_void_p), ("clips", C.c_void_p),
        ("call", C.c_void_p), ("score", C.c_void_p), ("indel_len", C.c_void_p),
        ("ins_str", C.c_void_p), ("ins_chars", C.c_void_p), ("ins_chars_cap", C.c_int64),
    ]


class pg_window(C.Structure):
    _fields_ = [("read_begin", C.c_int64), ("read_end", C.c_int64)]


class pg_kmer_edge(C.Structure):
    _fields_ = [
        ("key_hi", C.c_uint64), ("key_lo", C.c_uint64), ("window", C.c_int32), ("next", C.c_int8),
        ("alt", C.c_int8), ("pad_", C.c_int16), ("depth", C.c_int32), ("weight", C.c_int32),
    ]


class pg_serve_config(C.Structure):
    _fields_ = [
        ("device", C.c_int32), ("n_workers", C.c_int32), ("hbm_budget", C.c_int64), ("max_batch", C.c_int32),
        ("batched", C.c_int32), ("fix_snps", C.c_int32), ("fix_indels", C.c_int32), ("iupac", C.c_int32),
        ("diploid", C.c_int32), ("vcf_qe", C.c_int32), ("pad_", C.c_int32),
    ]


class pg_request(C.Structure):
    _fields_ = [("contig", C.c_int32), ("start", C.c_int32), ("stop", C.c_int32), ("pad_", C.c_int32)]


class pg_result(C.Structure):
    _fields_ = [
        ("status", C.c_int32), ("batch", C.c_int32), ("fasta", C.c_void_p), ("fasta_len", C.c_int64),
        ("changes", C.c_void_p), ("changes_len", C.c_int64), ("vcf", C.c_void_p), ("vcf_len", C.c_int64),
        ("message", C.c_char_p), ("queue_ms", C.c_double), ("run_ms", C.c_double), ("latency_ms", C.c_double),
        ("device_bytes", C.c_int64),
    ]


class pg_reassembly(C.Structure):
    _fields_ = [
        ("window", C.c_int32), ("is_gap", C.c_int32), ("region_start", C.c_int32), ("region_stop", C.c_int32),
        ("break_start", C.c_int32), ("break_stop", C.c_int32), ("break_radius", C.c_int32),
        ("fix_breaks", C.c_int32), ("gap_margin", C.c_int32), ("min_gap", C.c_int32),
        ("bases", C.c_void_p), ("orig", C.c_void_p),
    ]


class pg_reassembly_fix(C.Structure):
    _fields_ = [
        ("start", C.c_int32), ("status", C.c_int32), ("loop_len", C.c_int32), ("pad_", C.c_int32),
        ("was_off", C.c_int64), ("was_len", C.c_int64), ("patch_off", C.c_int64), ("patch_len", C.c_int64),
    ]


class pg_break(C.Structure):
    _fields_ = [("region", C.c_int32), ("start", C.c_int32), ("stop", C.c_int32), ("pad_", C.c_int32)]


# numpy dtype of pg_kmer_edge, for bulk views of edge arrays
def kmer_edge_dtype():
    import numpy as np
    return np.dtype([("key_hi", "<u8"), ("key_lo", "<u8"), ("window", "<i4"), ("next", "i1"), ("alt", "i1"),
                     ("pad_", "<i2"), ("depth", "<i4"), ("weight", "<i4")])


# numpy dtype of pg_change
def change_dtype():
    import numpy as np
    return np.dtype([("region", "<i4"), ("locus", "<i4"), ("call", "<u4"), ("indel_len", "<i4"), ("ins_str", "<i4"),
                     ("pad_", "<i4")])


# numpy dtype of pg_fix
def fix_dtype():
    import numpy as np
    return np.dtype([("locus", "<i4"), ("list", "<i4"), ("was_off", "<i8"), ("was_len", "<i8"),
                     ("patch_off", "<i8"), ("patch_len", "<i8")])


class pg_fix_options(C.Structure):
    _fields_ = [("fix_snps", C.c_int32), ("fix_indels", C.c_int32), ("iupac", C.c_int32), ("long_read", C.c_int32)]


# numpy dtype of pg_kmer_edge_wide (K <= 63)
def kmer_edge_wide_dtype():
    import numpy as np
    return np.dtype([("key0", "<u8"), ("key1", "<u8"), ("key2", "<u8"), ("key3", "<u8"), ("window", "<i4"),
                     ("next", "i1"), ("alt", "i1"), ("pad_", "<i2"), ("depth", "<i4"), ("weight", "<i4")])


def default_params(**kw):
    """Pilon's defaults (S/Pilon.scala:52-73); keyword overrides by field name."""
    p = pg_params(min_mq=0, min_qual=0, flank=10, default_qual=10, min_min_depth=5,
                  nonpf=0, duplicates=0, old_indel=0, fix_amb=0, long_read=0, bam_type=0,
                  long_read_only=0, min_depth=0.1)
    for k, v in kw.items():
        if not hasattr(p, k):
            raise AttributeError(k)
        setattr(p, k, v)
    return p


# Exported symbols of libpilon_gb300.so, one per declaration in the header.
EXPORTED = [
    "pg_open", "pg_close", "pg_last_error", "pg_default_params", "pg_version",
    "pg_set_reference", "pg_set_reads", "pg_set_reads_device", "pg_pileup_regions",
    "pg_fetch_stats", "pg_fetch_region", "pg_set_tuning", "pg_kmer_tally",
    "pg_last_kernel_ms", "pg_sync", "pg_phys_cov_scan_static", "pg_format_vcf", "pg_find_breaks",
    "pg_kmer_tally_breaks", "pg_fetch_all", "pg_graph_replays", "pg_last_tally_stats",
    "pg_find_duplications", "pg_kmer_tally_wide", "pg_kmer_tally_breaks_wide", "pg_fetch_changes",
    "pg_default_serve_config", "pg_serve_open", "pg_serve_submit", "pg_serve_poll", "pg_serve_release",
    "pg_serve_stats", "pg_serve_error", "pg_serve_close", "pg_kmer_tally_reads", "pg_reassemble",
    "pg_mark_deleted", "pg_set_reads_packed", "pg_region_fixes", "pg_changes_lines", "pg_scan_reads",
]

PG_STATIC_SCAN_MAX_POSITIONS = 16777216
