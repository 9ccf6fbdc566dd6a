"""The Rust binding crates (ffi/) against the C header, on the CPU.

No Rust toolchain exists in this image, so the crates cannot be compiled
here; this test pins their text instead:
* ffi/mczi-gpu-sys declares every function of include/mczi_gpu.h, in the same
  order, with the same arity and the Rust equivalent of every C type;
* its #[repr(C)] structs have the header's fields in the header's order;
* its constants equal the header's #defines;
* ffi/mczi-gpu exposes the reference's entry points with the reference's
  signatures (src/lib.rs:278-509, src/zi.rs:114, 152).
"""
import re
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "mczi_gpu.h"
SYS = ROOT / "ffi" / "mczi-gpu-sys" / "src" / "lib.rs"
SHIM = ROOT / "ffi" / "mczi-gpu" / "src" / "lib.rs"

SCALARS = {"int32_t": "i32", "uint32_t": "u32", "uint64_t": "u64", "uint8_t": "u8", "size_t": "usize",
           "float": "f32", "double": "f64", "char": "c_char", "void": "c_void", "int": "i32",
           "mczi_ctx": "mczi_ctx", "mczi_server": "mczi_server", "mczi_input": "mczi_input",
           "mczi_counter_config": "mczi_counter_config"}


def c_to_rust(t: str) -> str:
    """C parameter type -> Rust type, e.g. 'const char* const*' -> '*const *const c_char'."""
    t = t.replace("*", " * ").split()
    base_const = t[0] == "const"
    if base_const:
        t = t[1:]
    base, rest = t[0], t[1:]
    # pointer levels, innermost first: each '*' may be followed by 'const'
    levels = []
    i = 0
    while i < len(rest):
        assert rest[i] == "*", t
        const_after = i + 1 < len(rest) and rest[i + 1] == "const"
        levels.append(const_after)
        i += 2 if const_after else 1
    rust = SCALARS[base]
    pointee_const = base_const
    for const_after in levels:
        rust = ("*const " if pointee_const else "*mut ") + rust
        pointee_const = const_after
    return rust


def header_functions():
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    out = []
    for ret, name, args in re.findall(r"^\s*((?:const\s+)?\w+\**\s*\**)\s*(mczi_\w+)\s*\(([^;]*?)\);", text,
                                      flags=re.M | re.S):
        params = []
        for a in " ".join(args.split()).split(","):
            a = a.strip()
            m = re.match(r"(.*?)(\w+)$", a)
            params.append(c_to_rust(m.group(1).strip()))
        r = ret.strip()
        out.append((name, params, None if r == "void" else c_to_rust(r)))
    return out


def rust_functions():
    text = SYS.read_text()
    block = text[text.index('extern "C" {'):]
    out = []
    for name, args, ret in re.findall(r"pub fn (mczi_\w+)\((.*?)\)\s*(?:->\s*([^;]+))?;", block, flags=re.S):
        params = []
        for a in " ".join(args.split()).split(","):
            a = a.strip()
            if a:
                params.append(a.split(":", 1)[1].strip())
        out.append((name, params, ret.strip() if ret else None))
    return out


def test_every_header_function_is_bound_in_order():
    h = header_functions()
    r = rust_functions()
    assert [x[0] for x in r] == [x[0] for x in h]
    for (hn, hp, hr), (rn, rp, rr) in zip(h, r):
        assert len(hp) == len(rp), hn
        assert rp == hp, (hn, rp, hp)
        assert rr == hr, (hn, rr, hr)


def test_repr_c_structs_match_header():
    htext = HEADER.read_text()
    rtext = SYS.read_text()
    for name in ("mczi_counter_config", "mczi_input"):
        end = re.search(r"\}\s*" + name + ";", htext).start()
        body = htext[htext.rindex("typedef struct {", 0, end) + len("typedef struct {"):end]
        hfields = []
        for line in body.strip().splitlines():
            t, f = line.strip().rstrip(";").rsplit(None, 1)
            if f.startswith("*"):
                t, f = t + "*", f[1:]
            hfields.append((f, c_to_rust(t)))
        m2 = re.search(r"#\[repr\(C\)\]\s*#\[derive[^\]]*\]\s*pub struct " + name + r" \{(.*?)\}", rtext, flags=re.S)
        rfields = [(f.strip(), t.strip()) for f, t in re.findall(r"pub (\w+):\s*([^,]+),", m2.group(1))]
        assert rfields == hfields, name


def test_constants_match_header():
    h = dict(re.findall(r"#define (MCZI_\w+) \(?(-?\d+)\)?", HEADER.read_text()))
    r = dict(re.findall(r"pub const (MCZI_\w+): i32 = (-?\d+);", SYS.read_text()))
    assert r == h


def test_shim_keeps_reference_signatures():
    text = " ".join(SHIM.read_text().split())
    for sig in [
        "pub fn count_inputs(inputs: &[PathBuf], config: CounterConfig) -> Result<Vec<CountedKmer>>",
        "pub fn count_datasets(inputs: &[PathBuf], config: CounterConfig) -> Result<Vec<CountedKmer>>",
        "pub fn count_inputs_to_fasta_path(inputs: &[PathBuf], config: CounterConfig, output_path: &Path) -> Result<()>",
        "pub fn count_datasets_to_fasta_path(inputs: &[PathBuf], config: CounterConfig, output_path: &Path) -> Result<()>",
        "pub fn count_inputs_to_kff_path(inputs: &[PathBuf], config: CounterConfig, output_path: &Path) -> Result<()>",
        "pub fn count_datasets_to_kff_path(inputs: &[PathBuf], config: CounterConfig, output_path: &Path) -> Result<()>",
        "pub fn count_inputs_to_kmer_fasta_path(inputs: &[PathBuf], config: CounterConfig, output_path: &Path) "
        "-> Result<u64>",
        "pub fn count_datasets_to_kmer_fasta_path(inputs: &[PathBuf], config: CounterConfig, output_path: &Path) "
        "-> Result<u64>",
        "pub fn build_dictionary(index_path: &Path, k: usize, m: usize, _threads: usize, _ram_limit_gib: usize, "
        "_tmp_dir: &Path) -> Result<Dictionary>",
        "pub fn collect_query_kmers_absent_from_index(dictionary: &Dictionary, query_inputs: &[PathBuf]) "
        "-> Result<HashSet<EncodedKmer>>",
    ]:
        assert sig in text, sig
    # CounterConfig / CountedKmer mirror src/lib.rs:48-66 field for field
    assert "pub struct CounterConfig { pub k: usize, pub minimizer: usize, pub threshold: Count, " \
           "pub partition_count: usize, }" in text
    assert "pub struct CountedKmer { pub encoded: EncodedKmer, pub count: Count, }" in text


def test_type_mapping_examples():
    assert c_to_rust("const char* const*") == "*const *const c_char"
    assert c_to_rust("mczi_ctx**") == "*mut *mut mczi_ctx"
    assert c_to_rust("const mczi_ctx*") == "*const mczi_ctx"
    assert c_to_rust("uint8_t**") == "*mut *mut u8"
    assert c_to_rust("void*") == "*mut c_void"
