/*
 * pilon_gb300 — C ABI of the GB300 pileup / call / k-mer-tally engine.
 *
 * The engine replaces the per-read and per-position hot loops of Pilon 1.24
 * (broadinstitute/pilon).  Every entry point below names the reference code it
 * stands in for (paths are relative to the reference project root; S/ is
 * src/main/scala/org/broadinstitute/pilon/).
 *
 * Conventions
 *   - Plain C types only: pointers, sizes, POD structs.  No exceptions cross
 *     the boundary; every call returns a pg_status and pg_last_error() gives
 *     the message of the last failure on that context.
 *   - Input buffers are caller-owned.  Results stay in the context (device
 *     memory) until the next pg_pileup_regions / pg_kmer_tally call on the
 *     same context, and are copied out with the pg_fetch_* calls.
 *   - One context is used by one host thread at a time; all its work is
 *     ordered on the context's own CUDA stream.
 *   - Coordinates are Pilon's: 1-based, closed intervals (S/Region.scala:21-45).
 */
#ifndef PILON_GB300_H
#define PILON_GB300_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum pg_status {
  PG_OK = 0,
  PG_ERR_ARG = 1,        /* bad argument (null pointer, bad size, bad option) */
  PG_ERR_CUDA = 2,       /* CUDA runtime error; context should be closed */
  PG_ERR_NOMEM = 3,      /* device memory budget exceeded, or host memory or threads
                            could not be had (no C++ exception leaves a call) */
  PG_ERR_INDEX = 4,      /* an index left its array; the reference throws
                            ArrayIndexOutOfBoundsException here (indel left
                            shift below the region start,
                            S/PileUpRegion.scala:155-182) */
  PG_ERR_STATE = 5,      /* call out of order (e.g. fetch before process) */
  PG_ERR_LIMIT = 6,      /* a documented size limit was exceeded */
  PG_ERR_TIMEOUT = 7     /* a bounded device-side wait ran out */
} pg_status;

/* Long-read type of one BAM (S/BamFile.scala:32-47). */
enum { PG_NOT_LONG_READ = 0, PG_NANOPORE = 1, PG_PACBIO = 2 };
/* BAM type (S/BamFile.scala:29, S/Pilon.scala:130-231). */
enum { PG_BAM_FRAGS = 0, PG_BAM_JUMPS = 1, PG_BAM_UNPAIRED = 2, PG_BAM_BAM = 3 };

/* Options of the hot path, mirroring the global vars of S/Pilon.scala:28-73.
 * pg_default_params() fills in Pilon's defaults. */
typedef struct pg_params {
  int32_t min_mq;          /* --minmq, default 0 */
  int32_t min_qual;        /* --minqual, default 0 */
  int32_t flank;           /* --flank, default 10 */
  int32_t default_qual;    /* --defaultqual, default 10; a byte (-128..127) as in Pilon */
  int32_t min_min_depth;   /* constant 5 */
  int32_t nonpf;           /* --nonpf */
  int32_t duplicates;      /* --duplicates */
  int32_t old_indel;       /* --oldindel */
  int32_t fix_amb;         /* Pilon.iupac || Pilon.fixAmb (S/GenomeRegion.scala:235) */
  int32_t long_read;       /* PG_NOT_LONG_READ / PG_NANOPORE / PG_PACBIO of the BAM */
  int32_t bam_type;        /* PG_BAM_* of the BAM */
  int32_t long_read_only;  /* Pilon.longread && no frags BAM (S/GenomeRegion.scala:147) */
  double  min_depth;       /* --mindepth, default 0.1 */
} pg_params;

/* Aligned reads of one BAM as structure-of-arrays, in BAM (coordinate) order.
 * Field meanings follow the htsjdk SAMRecord getters used on the hot path
 * (S/PileUpRegion.scala:103-115, S/BamFile.scala:101-105, 137). */
typedef struct pg_reads {
  int64_t n_reads;
  const int32_t *pos;         /* getAlignmentStart, 1-based */
  const int32_t *aend;        /* getAlignmentEnd (pos + ref-consuming length - 1) */
  const uint16_t *flag;       /* SAM flag word */
  const uint8_t *mapq;        /* getMappingQuality */
  const int32_t *tlen;        /* getInferredInsertSize */
  const int32_t *ref_id;      /* getReferenceIndex */
  const int32_t *mate_ref_id; /* getMateReferenceIndex */
  const int64_t *cigar_off;   /* first CIGAR word of the read in `cigar` */
  const uint16_t *n_cigar;    /* number of CIGAR words */
  const uint32_t *cigar;      /* BAM CIGAR words: len << 4 | op (MIDNSHP=X -> 0..8) */
  const int64_t *seq_off;     /* first byte of the read in `seq` */
  const int32_t *l_seq;       /* getReadLength */
  const uint8_t *seq;         /* BAM 4-bit bases, two per byte, high nibble first,
                                 "=ACMGRSVTWYHKDBN" */
  const int64_t *qual_off;    /* first byte of the read in `qual` */
  const uint8_t *qual;        /* Phred bytes; a first byte of 0xFF means absent
                                 (getBaseQualities() is empty -> defaultQual) */
  int64_t n_cigar_words;      /* total length of `cigar` */
  int64_t seq_bytes;          /* total length of `seq` */
  int64_t qual_bytes;         /* total length of `qual` */
} pg_reads;

/* One region (GenomeRegion) and the reads fed to it.  The reads of
 * [read_begin, read_end) must contain every read of `contig` that overlaps
 * [max(start-10000,0), min(stop+10000,len)] (S/BamFile.scala:117-119); reads
 * outside that window inside the range are skipped by the engine, exactly as
 * the reference's query would not return them.  The range must hold reads of
 * `contig` only, in position order (it is searched by position): not the
 * neighbouring contigs' reads nor the unplaced reads (reference -1) at the end
 * of a coordinate-sorted store. */
typedef struct pg_region {
  int32_t contig;            /* index into the contigs given to pg_set_reference */
  int32_t start;             /* 1-based first base */
  int32_t stop;              /* 1-based last base, inclusive */
  int32_t pad_;
  int64_t read_begin;
  int64_t read_end;
} pg_region;

/* Per-region scalars (PileUpRegion / GenomeRegion / BamFile fields). */
typedef struct pg_region_stats {
  int64_t base_count;        /* PileUpRegion.baseCount */
  int64_t read_count;        /* PileUpRegion.readCount */
  int32_t phys_cov_start;    /* PileUpRegion.physCovStart */
  int32_t insert_size_start; /* PileUpRegion.insertSizeStart */
  int32_t min_depth;         /* GenomeRegion.minDepth after postProcess */
  int32_t n_changes;         /* entries of the change map after pass 1 */
  /* BamFile.addInsert deltas of this region (S/BamFile.scala:194-202) */
  int64_t fr_count, fr_sum, fr_sumsq;
  int64_t rf_count, rf_sum, rf_sumsq;
  int32_t error;             /* PG_ERR_INDEX when the reference would throw */
  int32_t n_ins_strings;     /* insertion-call strings of this region */
} pg_region_stats;

/* Call flags, one uint32 per position (PileUp.BaseCall, S/PileUp.scala:132-255,
 * and the pass-1 disposition of S/GenomeRegion.scala:237-272). */
#define PG_CALL_BASE(f)      ((f) & 3u)          /* baseIndex (A,C,G,T) */
#define PG_CALL_ALT(f)       (((f) >> 2) & 3u)   /* altBaseIndex */
#define PG_CALL_HAS_BASE     (1u << 4)           /* n > 0 (else base is 'N') */
#define PG_CALL_HOMO         (1u << 5)
#define PG_CALL_INS          (1u << 6)           /* insertion call */
#define PG_CALL_DEL          (1u << 7)           /* deletion call */
#define PG_CALL_HOMO_INDEL   (1u << 8)
#define PG_CALL_CHANGE(f)    (((f) >> 9) & 7u)   /* PG_CHANGE_* */
#define PG_CALL_CONFIRMED    (1u << 12)
#define PG_CALL_DELETED      (1u << 13)          /* inside a called deletion */
enum { PG_CHANGE_NONE = 0, PG_CHANGE_SNP = 1, PG_CHANGE_INS = 2, PG_CHANGE_DEL = 3, PG_CHANGE_AMB = 4 };

/* Host buffers for one region's results; every array has `size` entries
 * (count and qual_sum have 4*size, A,C,G,T interleaved per position).  Any
 * pointer may be NULL to skip that field. */
typedef struct pg_region_out {
  int32_t *count;            /* PileUp.baseCount */
  int64_t *qual_sum;         /* PileUp.qualSum */
  int32_t *mq_sum, *q_sum, *phys_cov, *insert_size, *bad_pair;
  int32_t *deletions, *del_qual, *insertions, *ins_qual, *clips;
  uint32_t *call;            /* PG_CALL_* flags */
  int64_t *score;            /* BaseCall.score */
  int32_t *indel_len;        /* length of the called insertion/deletion, else 0 */
  int32_t *ins_str;          /* offset of the called insertion in ins_chars, else -1 */
  char *ins_chars;           /* insertion-call characters (n_ins_strings total bytes
                                = sum of their lengths), may be NULL */
  int64_t ins_chars_cap;     /* capacity of ins_chars */
} pg_region_out;

/* One local-reassembly window for the k-mer tally: reads [read_begin,
 * read_end) of the read store are the window's recruited reads, in the order
 * Assembler.addReads sees them (S/GapFiller.scala:125-129). */
typedef struct pg_window {
  int64_t read_begin;
  int64_t read_end;
} pg_window;

/* One graph edge of Assembler.buildGraph (S/Assembler.scala:132-154):
 * kmer -> kmer[1:] + next; alt >= 0 adds the altGraph link kmer[1:] + alt.
 * The K-mer (K <= 32) is given as 4-bit BAM codes ("=ACMGRSVTWYHKDBN"), so
 * K-mers containing N or IUPAC codes are exact too: base j sits at bits
 * 60-4*(j%16) of key_hi (j < 16) or key_lo (j >= 16). */
typedef struct pg_kmer_edge {
  uint64_t key_hi;
  uint64_t key_lo;
  int32_t window;
  int8_t next;               /* called base index (A,C,G,T) */
  int8_t alt;                /* alt base index, or -1 when the call is homozygous */
  int16_t pad_;
  int32_t depth;             /* PileUp.depth of the K-mer */
  int32_t weight;            /* baseCount of the called base */
} pg_kmer_edge;

/* One graph edge for any K <= 63 (pg_kmer_tally_wide): the K-mer as 4-bit BAM
 * codes, base j at bits 60-4*(j%16) of key[j/16]; other fields as in
 * pg_kmer_edge. */
typedef struct pg_kmer_edge_wide {
  uint64_t key[4];
  int32_t window;
  int8_t next;
  int8_t alt;
  int16_t pad_;
  int32_t depth;
  int32_t weight;
} pg_kmer_edge_wide;

/* One break candidate of GenomeRegion.possibleBreaks (S/GenomeRegion.scala:
 * 659-720): contig loci start..stop (1-based, inclusive) in region `region`
 * of the last pg_pileup_regions call. */
typedef struct pg_break {
  int32_t region;
  int32_t start;
  int32_t stop;
  int32_t pad_;
} pg_break;

typedef struct pg_ctx pg_ctx;

/* ---- context ----------------------------------------------------------- */
/* Opens a context on CUDA device `device`.  Replaces nothing in the
 * reference (which has no device); allocates the context's stream.
 * PG_ERR_ARG when ctx is NULL.  When there is no such device (or the stream
 * cannot be made) it returns PG_ERR_CUDA and still sets *ctx, so that
 * pg_last_error can say why; calls that use the device then return
 * PG_ERR_STATE on it, and pg_close frees it. */
pg_status pg_open(pg_ctx **ctx, int device);
void pg_close(pg_ctx *ctx);
const char *pg_last_error(const pg_ctx *ctx);
/* Fills Pilon's defaults (S/Pilon.scala:52-73). */
void pg_default_params(pg_params *p);
/* Library version string. */
const char *pg_version(void);

/* ---- reference ----------------------------------------------------------
 * Replaces GenomeFile's contig load (S/GenomeFile.scala:30-42): raw FASTA
 * bytes per contig, uploaded once and kept resident. */
pg_status pg_set_reference(pg_ctx *ctx, int32_t n_contigs, const int64_t *lens,
                           const uint8_t *const *bases);

/* ---- reads --------------------------------------------------------------
 * The BAM read feed (S/BamFile.scala:108-139) as packed SoA.  Host pointers:
 * the arrays are copied into the context's device read store.  Device
 * pointers (pg_set_reads_device): used in place, must outlive their use. */
pg_status pg_set_reads(pg_ctx *ctx, const pg_reads *host_reads);
pg_status pg_set_reads_device(pg_ctx *ctx, const pg_reads *device_reads);
/* pg_set_reads for a packed store (each read's CIGAR words, base bytes and
 * qualities right after the previous read's, as a BAM decoder lays them out):
 * cigar_off, seq_off, qual_off and aend are not read (they may be NULL) but
 * derived on the device from n_cigar, l_seq and the CIGARs, so 28 bytes less
 * per read cross the host link.  PG_ERR_ARG when the lengths do not fill
 * n_cigar_words, seq_bytes and qual_bytes exactly. */
pg_status pg_set_reads_packed(pg_ctx *ctx, const pg_reads *host_reads);

/* ---- pileup + calls -------------------------------------------------------
 * For every region: BamFile.process + PileUpRegion.addRead
 * (S/BamFile.scala:108-148, S/PileUpRegion.scala:102-220), computePhysCov
 * (S/PileUpRegion.scala:90-100), PileUp.baseCall (S/PileUp.scala:132-257) and
 * pass 1 of GenomeRegion.postProcess (S/GenomeRegion.scala:214-272), including
 * the deletion-span update of later pileups.  `batched` = 0 launches the
 * kernels once per region (the plain path); 1 runs all regions in one
 * persistent launch per kernel.  PG_ERR_INDEX reports regions on which the
 * reference would throw; their pg_region_stats.error is set and the results
 * of all other regions remain available. */
pg_status pg_pileup_regions(pg_ctx *ctx, const pg_region *regions, int32_t n_regions,
                            const pg_params *params, int32_t batched);

/* Per-region scalars of the last pg_pileup_regions call. */
pg_status pg_fetch_stats(pg_ctx *ctx, int32_t region, pg_region_stats *stats);
/* Copies one region's arrays into caller host buffers. */
pg_status pg_fetch_region(pg_ctx *ctx, int32_t region, pg_region_out *out);
/* Copies the arrays of all regions of the last call at once: each array of
 * `out` holds sum(stop - start + 1) positions, the regions one after another
 * in call order (one copy per array instead of one per region). */
pg_status pg_fetch_all(pg_ctx *ctx, pg_region_out *out);

/* One change of pass 1 of GenomeRegion.postProcess (S/GenomeRegion.scala:
 * 233-272): a position whose call became a SNP, INS, DEL or AMB change after
 * the deletion-span update.  These are what identifyAndFixIssues turns into
 * fixes (S/GenomeRegion.scala:307-414). */
typedef struct pg_change {
  int32_t region;            /* region of the last pg_pileup_regions call */
  int32_t locus;             /* 1-based contig locus */
  uint32_t call;             /* PG_CALL_* flags: base, alt, change kind */
  int32_t indel_len;         /* inserted or deleted bases, else 0 */
  int32_t ins_str;           /* offset of the inserted bases in ins_chars, else -1 */
  int32_t pad_;
} pg_change;

/* The changes of every region of the last call, ordered by region and locus,
 * and the insertion characters they point into (copied when ins_chars is not
 * NULL and they fit in ins_cap).  *n_changes and *n_ins_chars receive the
 * full sizes; the changes are copied up to cap.  This is what the fix lists
 * need, a small fraction of the per-position arrays. */
pg_status pg_fetch_changes(pg_ctx *ctx, pg_change *out, int64_t cap, int64_t *n_changes, char *ins_chars,
                           int64_t ins_cap, int64_t *n_ins_chars);

/* ---- fix lists and the changes file (host only: no context or device) ----
 * One Fix of GenomeRegion (locus, was, patch): its strings are text[was_off ..
 * was_off + was_len) and text[patch_off .. patch_off + patch_len). */
typedef struct pg_fix {
  int32_t locus;             /* first replaced locus (1-based) */
  int32_t list;              /* 0: snpFixList, 1: smallFixList, 2: bigFixList */
  int64_t was_off, was_len;
  int64_t patch_off, patch_len;
} pg_fix;

/* The --fix switches that decide which changes become fixes. */
typedef struct pg_fix_options {
  int32_t fix_snps;          /* --fix snps (AMB changes too, as bases or with iupac as codes) */
  int32_t fix_indels;        /* --fix indels */
  int32_t iupac;             /* --iupac: an AMB change is fixed as its IUPAC code, in the small list */
  int32_t long_read;         /* long-read only: AMB changes are not fixed */
} pg_fix_options;

/* The fix lists of one region from its changes (the region's slice of
 * pg_fetch_changes), as GenomeRegion.identifyAndFixIssues builds them
 * (S/GenomeRegion.scala:307-380): SNP and AMB changes in snpFixList (AMB with
 * --iupac in smallFixList as a code, Bases.toIUPAC), insertions and deletions
 * in smallFixList, each list last change first, as the reference prepends;
 * `excluded` (NULL or one byte per region position) drops the changes that
 * excludeMotifs marks.  `contig` is the whole contig (a deletion may run past
 * the region).  bases_snp (region size bytes) receives the region's bases
 * after fixIssues(snpFixList) and bases (bases_cap bytes) those after
 * fixIssues(smallFixList) on top (S/GenomeRegion.scala:557-621).  The fixes,
 * snp list first, go to fixes with their strings in text.  *n_fixes,
 * *text_len and *bases_len receive the full sizes; PG_ERR_LIMIT when one of
 * them does not fit (nothing is copied then).  Reference bytes are ASCII. */
pg_status pg_region_fixes(const pg_change *changes, int64_t n_changes, const char *ins_chars, int64_t n_ins_chars,
                          const uint8_t *contig, int64_t contig_len, int32_t start, int32_t stop,
                          const pg_fix_options *opts, const uint8_t *excluded, pg_fix *fixes, int64_t fix_cap,
                          int64_t *n_fixes, char *text, int64_t text_cap, int64_t *text_len, uint8_t *bases_snp,
                          uint8_t *bases, int64_t bases_cap, int64_t *bases_len);

/* The changes file's lines of one region (S/GenomeRegion.scala:645-657):
 * fixFixList over the fixes in the order given (snpFixList ++ smallFixList ++
 * bigFixList), then per fix "name:from[-to] new_name:from[-to] was patch"
 * with "." for an empty string, the new loci shifted by `offset` (the length
 * change of the contig's earlier regions) and by the fixes before it.
 * *out_len receives the full size; PG_ERR_LIMIT when it exceeds cap. */
pg_status pg_changes_lines(const pg_fix *fixes, int64_t n_fixes, const char *text, int64_t text_len,
                           const char *name, const char *new_name, int64_t offset, char *out, int64_t cap,
                           int64_t *out_len);

/* Launch shape of the pileup walk kernel: tile width (positions per CTA,
 * a power of two in [256, 4096]), warps per CTA (1..16) and variant (lanes
 * per read: 0 = 32, 1 = 16, 2 = 8, 3 = 4); 0 / -1 keep the current value.  The host
 * package's autotuner picks these. */
pg_status pg_set_tuning(pg_ctx *ctx, int32_t tile_width, int32_t warps_per_cta, int32_t variant);

/* ---- k-mer tally ----------------------------------------------------------
 * Assembler.addRead/addToPileups for every window (S/Assembler.scala:55-87)
 * followed by buildGraph (S/Assembler.scala:132-154), K <= 32.  Returns the
 * edges of all windows; *n_edges receives the count (up to cap). */
pg_status pg_kmer_tally(pg_ctx *ctx, const pg_window *windows, int32_t n_windows,
                        int32_t K, const pg_params *params, int32_t min_depth,
                        pg_kmer_edge *edges, int64_t cap, int64_t *n_edges);
/* The same tally for 1 <= K <= 63, Pilon's default K = 47 included
 * (S/Assembler.scala:25), with 4-word K-mer keys in the edges.  K-mers of
 * A/C/G/T only are counted in tables of 2-bit keys (128 bits, inserted with a
 * 16-byte compare-and-swap); the others in tables of 4-bit keys. */
pg_status pg_kmer_tally_wide(pg_ctx *ctx, const pg_window *windows, int32_t n_windows,
                             int32_t K, const pg_params *params, int32_t min_depth,
                             pg_kmer_edge_wide *edges, int64_t cap, int64_t *n_edges);

/* The tally of pg_kmer_tally_wide over windows of listed reads: window w
 * holds reads[windows[w].read_begin .. windows[w].read_end) (indices into the
 * read store, in the order Assembler.addReads sees them), so a window can
 * hold the reads GapFiller.recruitReads collects (S/GapFiller.scala:364-402):
 * the reads overlapping the flanks of a break, which are not one index range
 * of the store, and their stray mates anywhere in it. */
pg_status pg_kmer_tally_reads(pg_ctx *ctx, const int64_t *reads, int64_t n_reads, const pg_window *windows,
                              int32_t n_windows, int32_t K, const pg_params *params, int32_t min_depth,
                              pg_kmer_edge_wide *edges, int64_t cap, int64_t *n_edges);

/* ---- local reassembly (host) ---------------------------------------------
 * One gap or break to reassemble: GapFiller.fillGap (is_gap = 1) or
 * GapFiller.fixBreak (is_gap = 0) of a GenomeRegion (S/GapFiller.scala:39-47),
 * walked over the K-mer graph of window `window` of the edges given to
 * pg_reassemble (the tally of GapFiller.recruitReads' reads). */
typedef struct pg_reassembly {
  int32_t window;            /* window of the edges that holds this break's reads */
  int32_t is_gap;            /* 1: a gap of Ns (fillGap); 0: a possible break (fixBreak) */
  int32_t region_start;      /* the GenomeRegion, 1-based loci, inclusive */
  int32_t region_stop;
  int32_t break_start;       /* the gap or break, 1-based loci, inclusive */
  int32_t break_stop;
  int32_t break_radius;      /* GapFiller.breakRadius (S/GapFiller.scala:357-362) */
  int32_t fix_breaks;        /* Pilon.fixBreaks (--fix breaks, --variant): an unjoined break gets
                                the partial fill of a gap (S/GapFiller.scala:76) */
  int32_t gap_margin;        /* Pilon.gapMargin (--gapmargin, default 100000): a closed gap whose
                                length differs from the gap's by more is not taken (S/GapFiller.scala:69-73) */
  int32_t min_gap;           /* Pilon.minGap (--mingap, default 10): the Ns a partial fill leaves at least
                                (S/GapFiller.scala:92) */
  const char *bases;         /* the region's bases after its SNP fixes (region size bytes) */
  const char *orig;          /* the region's original bases (region size bytes) */
} pg_reassembly;

/* BamFile.scan's pass over a read store (S/BamFile.scala:295-337) on host
 * threads (0 = all cores), for local reassembly; no context or device.  Of
 * the reads that pass validateRead and are mapped, addInsert (:194-202) adds
 * a proper pair's inferred insert size, or an unpaired read's length, when it
 * lies in (0, huge): stats receives count, sum and sum of squares (each square
 * a wrapping 32-bit Int) for FR, RF and unpaired, in that order (9 values).
 * strays receives the indices, in store order, of the reads MateMap files as
 * stray mates (paired, not proper, mate mapped, on a reference below
 * n_contigs or with its mate on one): the first-of-pair reads, then the
 * second-of-pair ones; *n_first and *n_second their counts.  PG_ERR_LIMIT when
 * they exceed stray_cap (stats are filled all the same). */
pg_status pg_scan_reads(const pg_reads *reads, const pg_params *params, int32_t n_contigs, int32_t huge,
                        int32_t threads, int64_t *stats, int64_t *strays, int64_t stray_cap, int64_t *n_first,
                        int64_t *n_second);

/* The fix of one pg_reassembly, GenomeRegion.Fix (locus, was, patch). */
typedef struct pg_reassembly_fix {
  int32_t start;             /* first locus of the fix; 0 when there is no solution */
  int32_t status;            /* PG_OK, or PG_ERR_INDEX where the reference's require(...) fails */
  int32_t loop_len;          /* length of the shortest K-mer loop the walk met (a tandem repeat), 0 if none */
  int32_t pad_;
  int64_t was_off, was_len;     /* the replaced bases (refSubString), in text */
  int64_t patch_off, patch_len; /* the new bases, in text */
} pg_reassembly_fix;

/* GapFiller.assembleAcrossBreak (S/GapFiller.scala:49-100) for every job, on
 * the host: the walk of Assembler.multiBridge from both sides of the break
 * over the window's graph (S/Assembler.scala:164-284), the joins of
 * breakJoins / properOverlap / trimPatch (S/GapFiller.scala:161-262), and for
 * gaps the partial fill from each side's consensus.  `edges` are the output of
 * pg_kmer_tally_reads (any order); K is Assembler.K.  Jobs run on `threads`
 * host threads (0 = all cores).  The fixes' strings are copied into `text`
 * when they fit in text_cap bytes; *text_len receives their total size either
 * way (PG_ERR_LIMIT when it does not fit).  Needs no context or device.
 * When host memory runs out the job's status (and the call's) is
 * PG_ERR_NOMEM; no C++ exception leaves the call.
 * Scala's Set of solutions is taken in insertion order, which is its order up
 * to four elements. */
pg_status pg_reassemble(const pg_kmer_edge_wide *edges, int64_t n_edges, int32_t K, const pg_reassembly *jobs,
                        int32_t n_jobs, int32_t threads, pg_reassembly_fix *fixes, char *text, int64_t text_cap,
                        int64_t *text_len);

/* ---- VCF ----------------------------------------------------------------
 * The per-position records of GenomeRegion.writeVcf / Vcf.writeRecord
 * (S/GenomeRegion.scala:623-643, S/Vcf.scala:74-176) for one region of the
 * last pg_pileup_regions call, formatted on the device.  `name` is the
 * contig name.  The text (no header, no <DUP> or reassembly records) is
 * copied into `out` when it fits in `cap` bytes; *n_bytes receives its size
 * either way (PG_ERR_LIMIT when it does not fit).  variants_only = 1 keeps
 * only records whose ALT is not "." (a delta for serving). */
pg_status pg_format_vcf(pg_ctx *ctx, int32_t region, const char *name, int32_t diploid, int32_t vcf_qe,
                        int32_t variants_only, char *out, int64_t cap, int64_t *n_bytes);

/* Marks loci first_locus .. first_locus + count - 1 of region `region` of the
 * last pg_pileup_regions call as deleted, as GenomeRegion.writeVcf does for
 * the bases a local-reassembly fix replaces before it writes their records
 * (S/GenomeRegion.scala:632-638): pg_format_vcf then writes them as records
 * inside a change (filter Del, no indel record after them). */
pg_status pg_mark_deleted(pg_ctx *ctx, int32_t region, int32_t first_locus, int32_t count);

/* ---- break candidates ---------------------------------------------------
 * GenomeRegion.possibleBreaks (S/GenomeRegion.scala:659-763) with
 * pctBadOverall (:99-114) and fragCoverage (:287-300) for every region of the
 * last pg_pileup_regions call, computed on the device from the resident
 * pileups: the windows local reassembly works on (S/GenomeRegion.scala:
 * 395-410).  `min_min_depth` is Pilon's --mindepth floor (5).  Breaks are
 * returned sorted by region, then start; *n_breaks receives the count (up to
 * cap).  Regions on which the reference threw (pg_region_stats.error) have
 * none. */
pg_status pg_find_breaks(pg_ctx *ctx, int32_t min_min_depth, pg_break *out, int64_t cap, int64_t *n_breaks);

/* GenomeRegion.duplicationEvents (S/GenomeRegion.scala:735-741) for every
 * region of the last pg_pileup_regions call, on the device: pass 2 of
 * postProcess, copyNumber = Math.round(smooth(fragCoverage, 200) / mean
 * fragCoverage) (S/GenomeRegion.scala:190-210, 274-283), then summaryRegions of
 * copyNumber > 1 with slop 2000, away from the region's ends, longer than
 * 10,000 bases: the <DUP> records of Vcf.writeDup (S/Vcf.scala:194-202).
 * Sorted by region, then start (pg_break records); *n_dups receives the count
 * (up to cap).  Regions without reads have none. */
pg_status pg_find_duplications(pg_ctx *ctx, pg_break *out, int64_t cap, int64_t *n_dups);

/* The K-mer tally of pg_kmer_tally over one window per break of
 * pg_find_breaks(min_min_depth), built on the device without a host round
 * trip: window k holds the reads of break k's contig that start in
 * [start - radius - S, stop + radius], S the longest alignment span of the
 * read store (every read overlapping [start - radius, stop + radius] and a
 * few that end before it).  This stands in for GapFiller's read recruitment
 * (S/GapFiller.scala:364-402) without mate rescue.  *n_windows receives the
 * number of breaks. */
pg_status pg_kmer_tally_breaks(pg_ctx *ctx, int32_t min_min_depth, int32_t radius, int32_t K,
                               const pg_params *params, int32_t min_depth, pg_kmer_edge *edges, int64_t cap,
                               int64_t *n_windows, int64_t *n_edges);
/* pg_kmer_tally_breaks for 1 <= K <= 63 (see pg_kmer_tally_wide). */
pg_status pg_kmer_tally_breaks_wide(pg_ctx *ctx, int32_t min_min_depth, int32_t radius, int32_t K,
                                    const pg_params *params, int32_t min_depth, pg_kmer_edge_wide *edges,
                                    int64_t cap, int64_t *n_windows, int64_t *n_edges);

/* ---- timing -------------------------------------------------------------
 * Milliseconds of the dominant (pileup walk) kernel in the last
 * pg_pileup_regions call, measured with CUDA events on the context stream,
 * and its launch count. */
pg_status pg_last_kernel_ms(pg_ctx *ctx, double *walk_ms, double *total_ms, int32_t *launches);
/* The last pg_kmer_tally / pg_kmer_tally_breaks call on this context: the
 * device time of its tally kernels (CUDA events on the context stream, table
 * clearing and host copies excluded), its K-mer events (2 (L - K) per read of
 * length L > K in a window), the distinct K-mers of all windows, the largest
 * batch's table bytes and the number of batches.  A measurement hook; no
 * counterpart in the reference. */
pg_status pg_last_tally_stats(pg_ctx *ctx, double *kernel_ms, int64_t *kmer_events, int64_t *distinct_kmers,
                              int64_t *max_batch_table_bytes, int32_t *batches);
/* Synchronises the context stream. */
pg_status pg_sync(pg_ctx *ctx);
/* Number of pg_pileup_regions calls on this context that replayed a recorded
 * CUDA graph instead of launching the kernels one by one.  A batched call is
 * recorded on its second identical occurrence and replayed after that while
 * the plan, the options and every buffer the graph uses stay the same; a call
 * that reallocates one of those buffers ends the replays until the next
 * recording.  No counterpart in the reference (a measurement hook). */
pg_status pg_graph_replays(pg_ctx *ctx, int32_t *replays);

/* ---- serving ------------------------------------------------------------
 * Region-polish requests with continuous batching.  A request is the work of
 * `pilon --targets contig:start-stop --fix snps,indels --vcf --changes` on one
 * region (S/GenomeFile.scala:215-250): GenomeRegion.processBam, postProcess,
 * identifyAndFixIssues and fixIssues (S/GenomeRegion.scala:214-414, 557-621),
 * writeChanges (:645-657) and Vcf.writeRecord (S/Vcf.scala:74-176).
 *
 * pg_serve_open uploads the reference and the read store once and keeps them
 * resident on the device; n_workers host threads each own an engine context
 * (own CUDA stream and buffers) over that store.  A free worker takes, from
 * the head of the queue, every request whose device bytes still fit
 * hbm_budget beside the batches already running (at most max_batch when it is
 * > 0) and runs them as one pg_pileup_regions call; requests arriving
 * meanwhile wait until memory and a worker free up, and the batches of
 * different workers overlap on the GPU.  A request's device bytes are 116 per
 * position of the region plus 16 per read of its query window (the pileup and
 * call records and per-read state of one call); a request needing more than
 * the whole budget is refused at submit with PG_ERR_NOMEM.  Each worker
 * context keeps its buffers between batches, and also holds event buffers
 * sized once from the store.
 *
 * Each answer holds the region's polished bases (no FASTA header or line
 * breaks), its changes-file lines (the target as its own output entry) and its
 * VCF records whose ALT is not "." (no header; no <DUP> records).  A target on
 * which the reference throws (PG_ERR_INDEX, see pg_pileup_regions) fails only
 * that request.  The server object is thread-safe. */
typedef struct pg_server pg_server;

typedef struct pg_serve_config {
  int32_t device;
  int32_t n_workers;       /* engine contexts working at once, 1..64 */
  int64_t hbm_budget;      /* device bytes the requests in flight may need together */
  int32_t max_batch;       /* most requests in one batch; 0 = no limit */
  int32_t batched;         /* 1: one batched launch per batch; 0: the plain per-region path */
  int32_t fix_snps;        /* --fix snps (with amb through pg_params.fix_amb) */
  int32_t fix_indels;      /* --fix indels */
  int32_t iupac;           /* --iupac */
  int32_t diploid;         /* --diploid */
  int32_t vcf_qe;          /* --vcfqe */
  int32_t pad_;
} pg_serve_config;

typedef struct pg_request {
  int32_t contig;          /* index into the contigs given to pg_serve_open */
  int32_t start, stop;     /* 1-based, inclusive */
  int32_t pad_;
} pg_request;

typedef struct pg_result {
  int32_t status;          /* PG_OK or this request's error */
  int32_t batch;           /* batch number it ran in, from 1 */
  const char *fasta;       /* polished bases of the region */
  int64_t fasta_len;
  const char *changes;     /* changes-file lines */
  int64_t changes_len;
  const char *vcf;         /* VCF records with an ALT */
  int64_t vcf_len;
  const char *message;     /* why the request failed, else "" */
  double queue_ms;         /* submit -> start of its batch */
  double run_ms;           /* start of its batch -> answered */
  double latency_ms;       /* submit -> answered */
  int64_t device_bytes;    /* the bytes it was admitted with */
} pg_result;

/* Fills the defaults: device 0, 2 workers, an 8 GiB budget, batched,
 * --fix snps,indels. */
void pg_default_serve_config(pg_serve_config *cfg);
/* Starts a server over one coordinate-sorted read store (host arrays, copied
 * to the device).  Like pg_open, *srv is set even on failure so that
 * pg_serve_error can say why; pg_serve_close frees it. */
pg_status pg_serve_open(pg_server **srv, const pg_serve_config *cfg, const pg_params *params, int32_t n_contigs,
                        const char *const *names, const int64_t *lens, const uint8_t *const *bases,
                        const pg_reads *host_reads);
/* Queues one request; *ticket identifies it. */
pg_status pg_serve_submit(pg_server *srv, const pg_request *req, uint64_t *ticket);
/* The request's answer: waits up to wait_ms (-1: until answered); returns
 * PG_ERR_STATE when it is not answered yet.  The strings stay valid until
 * pg_serve_release of the ticket. */
pg_status pg_serve_poll(pg_server *srv, uint64_t ticket, int32_t wait_ms, pg_result *out);
/* Frees an answered request's result. */
pg_status pg_serve_release(pg_server *srv, uint64_t ticket);
/* Batches run so far, device bytes of the requests in flight and their peak. */
pg_status pg_serve_stats(pg_server *srv, int64_t *batches, int64_t *in_flight_bytes, int64_t *peak_in_flight_bytes);
const char *pg_serve_error(const pg_server *srv);
/* Answers every queued request, then stops the workers and frees the server. */
void pg_serve_close(pg_server *srv);

/* ---- physical-coverage scan without device allocation ----------------------
 * This entry point has no counterpart in the reference.  It is for callers
 * that cannot let a library allocate device memory: a host whose own pool
 * (a JVM allocator, a PyTorch caching allocator) already holds the device's
 * memory, where a cudaMalloc could fail, fragment the pool or synchronise.
 *
 * It turns one region's physical-coverage and insert-size difference arrays
 * (caller device buffers of n_positions int32 each, the +1/-1 and +size/-size
 * updates of physCovIncr) into the prefix-summed values of computePhysCov,
 * starting from the region's carry (physCovStart, insertSizeStart), and
 * divides insert size by coverage where coverage > 0.  Output may alias input.
 * Work is queued on `stream` (a cudaStream_t; NULL = legacy default stream);
 * the call does not synchronise.
 *
 * Its only scratch is a fixed 128 KiB device array inside the library, so it
 * allocates nothing; n_positions above PG_STATIC_SCAN_MAX_POSITIONS returns
 * PG_ERR_LIMIT.  The first call on each device looks up that array's device
 * address (make it before any stream capture) and keeps it for the life of the
 * process; a host that destroys the device's primary context (cudaDeviceReset)
 * must not call this entry point afterwards.  All calls share the array:
 * calls that overlap on the GPU race and must be serialised by the caller.
 * On failure a message is written to errbuf (may be NULL). */
#define PG_STATIC_SCAN_MAX_POSITIONS 16777216
pg_status pg_phys_cov_scan_static(const int32_t *phys_diff, const int32_t *insert_diff, int64_t n_positions,
                                  int32_t phys_cov_start, int32_t insert_size_start, int32_t *phys_cov,
                                  int32_t *insert_size, void *stream, char *errbuf, int32_t errcap);

#ifdef __cplusplus
}
#endif
#endif /* PILON_GB300_H */
