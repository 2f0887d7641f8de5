// slemm.cpp — the `slemm` command line over libslemm_gb300 (the GPU engine of this package).
//
// A drop-in for the reference program's user-level contract on the REML / prediction path:
// the same long options with getopt_long abbreviations, short letters and defaults
// (src/option.cpp:53-117, docs/options.md:43-142), the same CSV phenotype / covariate / SNP-info
// inputs and PLINK .bed/.bim/.fam genotypes (src/input.cpp:25-454), and the same output files:
// .reml.py.txt, .reml.snp.csv, .reml.blue.csv, .reml.vc.csv (src/output.cpp:4-82), .gstat.txt
// (src/output.cpp:85-120) and the GEBV csv of --prediction (src/pred.cpp:4-141).  The analyses run
// through the library's C ABI on one GPU: marker QC, DF-REML (--lrt), MC-REML, --iter_weighting,
// --lmm quadratic forms, --wls and GEBV.  Numbers are written with C++ stream defaults (six
// significant digits), as the reference writes them.
//
// Error behaviour follows the reference: problems found while reading input files print a message
// and exit with status 1; errors of the analysis print to stderr and the run ends normally.
//
// Options beyond the reference's: --gpu_device N (default 0), --gpu_precision
// fp16x2|bf16x2|bf16x3|fp32 (default fp16x2, the column-scaled FP16 hi+lo products),
// --gpu_autotune (split-K counts and ring plans of the packed products timed at first use) and
// --gpu_lanczos_reorth (reorthogonalised Lanczos seeds instead of the reference's recurrence).
#include "slemm_gpu.h"

#include <getopt.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <ctime>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <map>
#include <set>
#include <sstream>
#include <string>
#include <utility>
#include <vector>

namespace {

// An analysis error: printed to stderr by main, like the reference's thrown messages.
struct Failure {
  std::string msg;
};
[[noreturn]] void fail(const std::string& msg) { throw Failure{msg}; }
// An input-file error: printed and the program exits with status 1, as the reference's readers do.
[[noreturn]] void die(const std::string& msg)
{
  std::cout << msg << std::endl;
  std::exit(1);
}

void check(int status)
{
  if (status != SLEMM_OK) fail(std::string("\nError: ") + slemm_gpu_last_error() + "\n");
}

constexpr char kDelim = ',';

std::vector<std::string> split(const std::string& s, char d)
{
  std::vector<std::string> out;
  std::string item;
  std::stringstream ss(s);
  while (std::getline(ss, item, d)) out.push_back(item);
  return out;
}

void strip_cr(std::string& line)
{
  if (!line.empty() && line.back() == '\r') line.pop_back();
}

bool file_exists(const std::string& f)
{
  std::ifstream ifs(f);
  return ifs.good();
}

// Column of `name` in a CSV header (first column is the ID and never matches); −1 for an empty
// name; a name that is absent ends the run.
int header_col(const std::string& name, const std::vector<std::string>& header, const std::string& file)
{
  if (name.empty()) return -1;
  for (size_t i = 1; i < header.size(); ++i)
    if (header[i] == name) return (int)i;
  die(name + " not found in the header of " + file);
}

// A data line must have the header's fields (a trailing delimiter may drop the last, empty one).
void check_fields(const std::string& line, const std::vector<std::string>& cols, size_t nh, const std::string& file)
{
  if (!(cols.size() == nh || (!line.empty() && line.back() == kDelim && nh == cols.size() + 1)))
    die("\nError: " + line + " in " + file);
}

struct CsvFile {
  std::vector<std::string> header;
  std::vector<std::pair<std::string, std::vector<std::string>>> rows;   // (line, fields)
};

CsvFile read_csv(const std::string& file)
{
  std::ifstream ifs(file);
  if (!ifs.is_open()) die("Cannot open " + file);
  CsvFile f;
  std::string line;
  std::getline(ifs, line);
  strip_cr(line);
  f.header = split(line, kDelim);
  while (std::getline(ifs, line)) {
    strip_cr(line);
    std::vector<std::string> cols = split(line, kDelim);
    check_fields(line, cols, f.header.size(), file);
    f.rows.push_back({line, std::move(cols)});
  }
  return f;
}

bool has_value(const std::vector<std::string>& cols, int c) { return c >= 0 && (int)cols.size() > c && !cols[c].empty(); }

// Phenotype file: ID → (trait value, error-variance weight, 1 when no weight column is named).
std::map<std::string, std::pair<float, float>> read_phenotypes(const std::string& file, const std::string& trait,
                                                               const std::string& weight)
{
  CsvFile f = read_csv(file);
  const int tc = header_col(trait, f.header, file);
  const int wc = header_col(weight, f.header, file);
  std::map<std::string, std::pair<float, float>> out;
  for (auto& [line, cols] : f.rows) {
    if (wc < 0) {
      if (has_value(cols, tc)) out[cols[0]] = {std::stof(cols[tc]), 1.0f};
    } else if (has_value(cols, wc) && has_value(cols, tc)) {
      out[cols[0]] = {std::stof(cols[tc]), std::stof(cols[wc])};
    }
  }
  return out;
}

// Covariate file: ID → covariate values (rows with any named covariate empty are left out);
// with no covariates named every ID gets the intercept and the name list becomes {"intercept"}.
std::map<std::string, std::vector<float>> read_covariates(const std::string& file, std::vector<std::string>& names)
{
  CsvFile f = read_csv(file);
  std::map<std::string, int> col_of;
  std::cout << "Header in covariate file: " << std::endl;
  for (size_t i = 1; i < f.header.size(); ++i) {
    std::cout << " " << f.header[i];
    col_of[f.header[i]] = (int)i;
  }
  std::cout << std::endl << "Covariates in command line option: " << std::endl;
  std::vector<int> cc;
  for (const auto& nm : names) {
    std::cout << " " << nm;
    auto it = col_of.find(nm);
    if (it == col_of.end()) die("\n" + nm + " not in covariate file");
    cc.push_back(it->second);
  }
  std::cout << std::endl;
  std::map<std::string, std::vector<float>> out;
  for (auto& [line, cols] : f.rows) {
    if (cc.empty()) {
      out[cols[0]] = {1.0f};
      continue;
    }
    std::vector<float> v;
    bool ok = true;
    for (int c : cc) {
      if (!has_value(cols, c)) {
        ok = false;
        break;
      }
      v.push_back(std::stof(cols[c]));
    }
    if (ok) out[cols[0]] = std::move(v);
  }
  if (cc.empty()) names.push_back("intercept");
  return out;
}

// SNP info file: SNP → (group, weight); group "NULL" and weight 1 unless columns are named.
std::map<std::string, std::pair<std::string, float>> read_snp_info(const std::string& file, const std::string& group,
                                                                   const std::string& weight)
{
  CsvFile f = read_csv(file);
  const int gc = header_col(group, f.header, file);
  const int wc = header_col(weight, f.header, file);
  std::map<std::string, std::pair<std::string, float>> out;
  for (auto& [line, cols] : f.rows) {
    if (gc < 0) {
      if (wc < 0) out[cols[0]] = {"NULL", 1.0f};
      else if (has_value(cols, wc)) out[cols[0]] = {"NULL", std::stof(cols[wc])};
    } else if (has_value(cols, gc)) {
      if (wc < 0) out[cols[0]] = {cols[gc], 1.0f};
      else if (has_value(cols, wc)) out[cols[0]] = {cols[gc], std::stof(cols[wc])};
    }
  }
  return out;
}

// .fam: within-family IDs in file order (lines shorter than 3 characters are skipped).
std::vector<std::string> read_fam(const std::string& file)
{
  std::ifstream ifs(file);
  if (!ifs.is_open()) die("Cannot open " + file);
  std::vector<std::string> ids;
  std::string line, fid, iid;
  while (std::getline(ifs, line)) {
    if (line.size() < 3) continue;
    std::stringstream ss(line);
    ss >> fid >> iid;
    ids.push_back(iid);
  }
  return ids;
}

struct BimRow {
  std::string chr, snp, a1, a2;
  int pos = 0;
};

std::vector<BimRow> read_bim(const std::string& file)
{
  std::ifstream ifs(file);
  if (!ifs.is_open()) die("Cannot open " + file);
  std::vector<BimRow> rows;
  std::string cm;
  while (ifs) {
    BimRow r;
    ifs >> r.chr;
    if (ifs.eof()) break;
    ifs >> r.snp >> cm >> r.pos >> r.a1 >> r.a2;
    rows.push_back(r);
  }
  return rows;
}

// The packed rows (after the 3-byte header, taken unchecked) of the .bed SNPs `pick` (indices into
// the .bim), each ⌈n_fam/4⌉ bytes, in that order.
std::vector<uint8_t> read_bed_rows(const std::string& file, int64_t n_fam, int64_t m_bim, const std::vector<int64_t>& pick)
{
  std::ifstream ifs(file, std::ios::binary);
  if (!ifs.is_open()) die("Cannot open " + file);
  const int64_t rb = (n_fam + 3) / 4;
  std::vector<uint8_t> out((size_t)pick.size() * rb);
  for (size_t r = 0; r < pick.size(); ++r) {
    if (pick[r] >= m_bim) fail("\nError: problem with the BED file. Has the FAM/BIM file been changed?\n");
    ifs.seekg(3 + pick[r] * rb);
    ifs.read(reinterpret_cast<char*>(out.data() + r * rb), rb);
    if (!ifs) fail("\nError: problem with the BED file. Has the FAM/BIM file been changed?\n");
  }
  return out;
}

// P(χ²₁ > x) = erfc(√(x/2)); 1 for x ≤ 0.
double chisq1_pval(double x) { return x <= 0 ? 1.0 : std::erfc(std::sqrt(x / 2.0)); }

float beta_pdf(float a, float b, float x)
{
  if (x <= 0.0f || x >= 1.0f) return 0.0f;
  return (float)(std::pow(x, a - 1.0) * std::pow(1.0 - x, b - 1.0));
}

std::string fmt(double v)
{
  std::ostringstream os;
  os << v;
  return os.str();
}

// A row of covariates as an Eigen row vector prints: each value right-aligned to the widest one,
// separated by single spaces.
std::string aligned_row(const std::vector<float>& v)
{
  std::vector<std::string> s;
  size_t w = 0;
  for (float x : v) {
    std::ostringstream os;
    os << x;
    s.push_back(os.str());
    w = std::max(w, s.back().size());
  }
  std::string out;
  for (size_t i = 0; i < s.size(); ++i) {
    if (i) out += ' ';
    out += std::string(w - s[i].size(), ' ') + s[i];
  }
  return out;
}

struct Markers {
  std::vector<std::string> names, groups;    // in analysis order
  std::vector<int64_t> bim_idx;              // .bim row of each
  std::vector<std::string> group_order;      // groups kept, in the order the markers are
  std::vector<int64_t> group_size;
  std::map<std::string, float> maf, hwep;
  std::vector<float> weight;                 // per marker, the SNP-info (or beta-pdf) weight
};

struct Inputs {
  std::vector<std::string> indi;             // kept individuals in .fam order
  std::vector<int64_t> keep_idx;             // their .fam positions
  int64_t n_fam = 0;
  std::vector<float> y, r, X;                // X: n × c column-major
  std::vector<std::string> covar_names;
  std::vector<BimRow> bim;
};

void write_reml(const std::string& prefix, const Inputs& in, const Markers& mk, const std::vector<float>& Py,
                const std::vector<float>& snp_blup, const std::vector<float>& blue, const std::vector<float>& var_blue,
                float vg, float ve, float lrt)
{
  const size_t n = in.indi.size(), c = in.covar_names.size();
  std::map<std::string, const BimRow*> bim_of;
  for (const auto& b : in.bim) bim_of[b.snp] = &b;
  std::ofstream ofs(prefix + ".reml.py.txt");
  ofs << "IID Py";
  for (const auto& nm : in.covar_names) ofs << ' ' << nm;
  ofs << " R\n";
  std::vector<float> row(c);
  for (size_t i = 0; i < n; ++i) {
    for (size_t j = 0; j < c; ++j) row[j] = in.X[j * n + i];
    ofs << in.indi[i] << ' ' << Py[i] << ' ' << aligned_row(row) << ' ' << in.r[i] << "\n";
  }
  ofs.close();
  ofs.open(prefix + ".reml.snp.csv");
  ofs << "SNP,Chr,Pos,Allele1,Allele2,MAF,HWE_Pval,Group,Weight,Effect" << std::endl;
  for (size_t k = 0; k < mk.names.size(); ++k) {
    const std::string& s = mk.names[k];
    const BimRow* b = bim_of[s];
    ofs << s << ',' << b->chr << ',' << b->pos << ',' << b->a1 << ',' << b->a2 << ',' << mk.maf.at(s) << ','
        << mk.hwep.at(s) << ',' << mk.groups[k] << ',' << 1 << ',' << snp_blup[k] << std::endl;
  }
  ofs.close();
  ofs.open(prefix + ".reml.blue.csv");
  if (lrt == 0) {
    ofs << "covar,blue\n";
    for (size_t i = 0; i < c; ++i) ofs << in.covar_names[i] << ',' << blue[i] << "\n";
  } else {
    ofs << "covar,blue,se,pval";
    for (const auto& nm : in.covar_names) ofs << ',' << nm;
    ofs << "\n";
    for (size_t i = 0; i < c; ++i) {
      const float vii = var_blue[i * c + i];
      ofs << in.covar_names[i] << ',' << blue[i] << ',' << std::sqrt(vii) << ','
          << chisq1_pval(blue[i] * blue[i] / vii);
      for (size_t j = 0; j < c; ++j) ofs << ',' << var_blue[j * c + i];
      ofs << "\n";
    }
  }
  ofs.close();
  int64_t num_markers = 0;
  for (int64_t s : mk.group_size) num_markers += s;
  ofs.open(prefix + ".reml.vc.csv");
  ofs << "pop_size," << n << std::endl;
  ofs << "num_markers," << num_markers << std::endl;
  ofs << "Vg," << vg << std::endl;
  ofs << "Ve," << ve << std::endl;
  ofs << "h2," << vg / (vg + ve) << std::endl;
  ofs << "LRT," << lrt << std::endl;
  ofs << "pval," << chisq1_pval(lrt) << std::endl;
}

void write_gstat(const std::string& prefix, const Inputs& in, const Markers& mk, int window_size, float vg,
                 const std::vector<int64_t>& var, const std::vector<float>& xPy, const std::vector<float>& xPx,
                 const std::vector<float>& xBx, const std::vector<float>& xSx)
{
  std::map<std::string, const BimRow*> bim_of;
  for (const auto& b : in.bim) bim_of[b.snp] = &b;
  const int64_t pop = (int64_t)in.indi.size();
  std::ofstream ofs(prefix + ".gstat.txt");
  ofs << "variant\tChr\tPos\tMAC\tMAF\tHWEP\txPy\txPx\txBx\txSx\tWindowSize\tChiSq\tPval" << std::endl;
  for (size_t q = 0; q < var.size(); ++q) {
    const std::string& s = mk.names[var[q]];
    const float maf = mk.maf.at(s);
    const BimRow* b = bim_of[s];
    const float chisq = (xPy[q] * xPy[q]) / (vg * xPx[q]);
    ofs << s << "\t" << b->chr << "\t" << b->pos << "\t" << int(maf * 2 * pop + 0.5) << "\t" << maf << "\t"
        << mk.hwep.at(s) << "\t" << xPy[q] << "\t" << xPx[q] << "\t" << xBx[q] << "\t" << xSx[q] << "\t" << window_size
        << "\t" << chisq << "\t" << chisq1_pval(chisq) << std::endl;
  }
}

int precision_code(const std::string& p)
{
  if (p == "fp16x2") return SLEMM_PREC_FP16X2;
  if (p == "bf16x2") return SLEMM_PREC_BF16X2;
  if (p == "bf16x3") return SLEMM_PREC_BF16X3;
  if (p == "fp32") return SLEMM_PREC_FP32;
  fail("\nError: --gpu_precision must be fp16x2, bf16x2, bf16x3 or fp32.\n");
}

// GEBV of every .fam individual from a .reml.snp.csv (src/pred.cpp:4-141): SNP effects per A2
// allele, flipped where the prediction .bim's allele 1 differs from the estimate's.
void run_prediction(const std::string& est_file, const std::string& bfile, const std::string& out_file, int device)
{
  std::ifstream ifs(est_file);
  if (!ifs.is_open()) die("Cannot open " + est_file);
  std::cout << "Reading SNP ESTIMATE file from [" + est_file + "]." << std::endl;
  std::string line;
  std::getline(ifs, line);
  std::map<std::string, std::pair<double, std::string>> eff;
  while (std::getline(ifs, line)) {
    std::vector<std::string> cols = split(line, ',');
    if (cols.size() < 10 || cols[0].empty() || cols[9].empty()) continue;
    eff[cols[0]] = {std::stod(cols[9]), cols[3]};
  }
  std::cout << "Reading PLINK FAM file from [" + bfile + ".fam]." << std::endl;
  const std::vector<std::string> fam = read_fam(bfile + ".fam");
  std::cout << "Reading PLINK BIM file from [" + bfile + ".bim]." << std::endl;
  const std::vector<BimRow> bim = read_bim(bfile + ".bim");
  std::vector<int64_t> pick;
  std::vector<double> alpha;
  std::vector<uint8_t> flip;
  for (size_t j = 0; j < bim.size(); ++j) {
    auto it = eff.find(bim[j].snp);
    if (it == eff.end()) continue;
    pick.push_back((int64_t)j);
    alpha.push_back(it->second.first);
    flip.push_back(bim[j].a1 != it->second.second ? 1 : 0);
  }
  if (pick.empty()) fail("\nNo SNPs found both in estimate file and in genotype file.\n");
  const int64_t n_fam = (int64_t)fam.size();
  std::cout << "Reading PLINK BED file from [" + bfile + ".bed] in SNP-major format..." << std::endl;
  const std::vector<uint8_t> rows = read_bed_rows(bfile + ".bed", n_fam, (int64_t)bim.size(), pick);
  check(slemm_gpu_init(device));
  slemm_geno* G = nullptr;
  check(slemm_gpu_genotype_create(rows.data(), n_fam, (int64_t)pick.size(), (n_fam + 3) / 4, nullptr, n_fam, 0, &G));
  std::vector<double> tgv(n_fam);
  const int st = slemm_gpu_gebv(G, alpha.data(), flip.data(), tgv.data());
  slemm_gpu_genotype_destroy(G);
  check(st);
  std::ofstream ofs(out_file);
  ofs << "IID,GEBV\n";
  for (int64_t i = 0; i < n_fam; ++i) ofs << fam[i] << ',' << tgv[i] << "\n";
}

void print_help() { printf("\nPlease see online documentation at https://github.com/jiang18/slemm\n"); }

void run(int argc, char** argv)
{
  if (argc < 3) {
    print_help();
    std::exit(1);
  }
  bool pred = false, reml = false, lmm = false, wls = false, lrt = false, iter_weighting = false, fake_geno = false;
  bool using_nr = false, using_ws = false;
  float sig_chisq = 1e6f, indep_r2 = 0.5f, max_h2 = 0.7f, min_maf = 0.f, rel_tol = 5e-4f, min_hwep = 0.f;
  int seed = 0, num_rand = 30, window_size = 1000, num_qf = 30, num_threads = 1, hwe_midp = 0, device = 0;
  bool gpu_autotune = false, gpu_reorth = false;
  unsigned subset_size = 1000;
  std::pair<float, float> beta_params{1.f, 1.f};
  std::string est_file, phen_file, trait, err_weight, covar_file, covar_names_str, snp_info, snp_group, snp_weight,
      bfile, out_file, precision = "fp16x2";
  static struct option opts[] = {
      {"min_hwe_pval", required_argument, 0, 'i'},    {"hwe_midp", no_argument, 0, 'H'},
      {"prediction", no_argument, 0, 'P'},            {"snp_estimate_file", required_argument, 0, 'a'},
      {"beta_weight_parameters", required_argument, 0, 'w'}, {"min_maf", required_argument, 0, 'j'},
      {"phenotype_file", required_argument, 0, 'p'},  {"trait_name", required_argument, 0, 't'},
      {"error_weight_name", required_argument, 0, 'e'}, {"covariate_file", required_argument, 0, 'c'},
      {"covariate_names", required_argument, 0, 'v'}, {"snp_info_file", required_argument, 0, 'm'},
      {"snp_set_name", required_argument, 0, 'x'},    {"snp_weight_name", required_argument, 0, 'y'},
      {"binary_genotype_file", required_argument, 0, 'g'}, {"bfile", required_argument, 0, 'b'},
      {"num_threads", required_argument, 0, 'u'},     {"output_file", required_argument, 0, 'o'},
      {"subset_size", required_argument, 0, 'z'},     {"rel_tol", required_argument, 0, 'r'},
      {"reml", no_argument, 0, 'R'},                  {"num_random_vectors", required_argument, 0, 'k'},
      {"lmm", no_argument, 0, 'L'},                   {"num_qf_markers", required_argument, 0, 'f'},
      {"window_size", required_argument, 0, 'q'},     {"max_heritability", required_argument, 0, 'h'},
      {"fake_geno", no_argument, 0, 'F'},             {"seed", required_argument, 0, 'd'},
      {"wls", no_argument, 0, 'S'},                   {"lrt", no_argument, 0, 'T'},
      {"iter_weighting", no_argument, 0, 'I'},        {"sig_chisq", required_argument, 0, 's'},
      {"indep_r2", required_argument, 0, 'n'},        {"gpu_device", required_argument, 0, 'D'},
      {"gpu_precision", required_argument, 0, 'G'},   {"gpu_autotune", no_argument, 0, 'A'},
      {"gpu_lanczos_reorth", no_argument, 0, 'O'},    {0, 0, 0, 0}};
  int idx = 0, opt;
  while ((opt = getopt_long(argc, argv, "HPRLFSTIAOi:a:w:j:p:t:e:c:v:m:x:y:g:b:u:o:z:r:k:f:q:h:d:s:n:D:G:", opts,
                            &idx)) != -1) {
    if (opt == '?' || opt == ':') {
      print_help();
      std::exit(1);
    }
    const char* name = opts[idx].name;
    if (optarg) printf("OPTION %s with ARG %s\n", name, optarg);
    else printf("OPTION %s initialized\n", name);
    switch (opt) {
      case 'i': min_hwep = std::stof(optarg); break;
      case 'H': hwe_midp = 1; break;
      case 'w': {
        const std::vector<std::string> v = split(optarg, ',');
        if (v.size() != 2) fail("\nError: incorrect option for beta weight.\n");
        beta_params = {std::stof(v[0]), std::stof(v[1])};
        break;
      }
      case 'j': min_maf = std::stof(optarg); break;
      case 'P': pred = true; break;
      case 'a': est_file = optarg; break;
      case 'p': phen_file = optarg; break;
      case 't': trait = optarg; break;
      case 'e': err_weight = optarg; break;
      case 'c': covar_file = optarg; break;
      case 'v': covar_names_str = optarg; break;
      case 'm': snp_info = optarg; break;
      case 'x': snp_group = optarg; break;
      case 'y': snp_weight = optarg; break;
      case 'g':
      case 'b': bfile = optarg; break;
      case 'u': num_threads = std::stoi(optarg); break;
      case 'o': out_file = optarg; break;
      case 'z': subset_size = (unsigned)std::stoi(optarg); break;
      case 'r': rel_tol = std::stof(optarg); break;
      case 'R': reml = true; break;
      case 'k':
        num_rand = std::stoi(optarg);
        using_nr = true;
        break;
      case 'L': lmm = true; break;
      case 'f': num_qf = std::stoi(optarg); break;
      case 'q':
        window_size = (int)std::stof(optarg);
        using_ws = true;
        break;
      case 'h': max_h2 = std::stof(optarg); break;
      case 'F': fake_geno = true; break;
      case 'd': seed = std::stoi(optarg); break;
      case 'S': wls = true; break;
      case 'T': lrt = true; break;
      case 'I': iter_weighting = true; break;
      case 's': sig_chisq = std::stof(optarg); break;
      case 'n': indep_r2 = std::stof(optarg); break;
      case 'D': device = std::stoi(optarg); break;
      case 'G': precision = optarg; break;
      case 'A': gpu_autotune = true; break;
      case 'O': gpu_reorth = true; break;
      default:
        print_help();
        std::exit(1);
    }
  }
  if (!(pred || reml || lmm || wls)) fail("\nError: --lmm OR --reml OR --pred OR --wls is missing.\n");
  if (pred) {
    std::cout << "Calculating total genetic values." << std::endl;
    if (bfile.empty()) fail("\nError: --binary_genotype_file is required for analysis.\n");
    if (est_file.empty()) fail("\nError: --snp_estimate_file is required for analysis.\n");
    if (out_file.empty()) fail("\nError: --output_file is required for analysis.\n");
    if (!(file_exists(bfile + ".fam") && file_exists(bfile + ".bim") && file_exists(bfile + ".bed")))
      fail("\nError: bed/bim/fam fileset NOT found.\n");
    run_prediction(est_file, bfile, out_file, device);
    std::cout << "Calculation of total genetic values finished." << std::endl;
    return;
  }
  if (phen_file.empty()) fail("\nError: --phenotype_file is required for analysis.\n");
  if (trait.empty()) fail("\nError: --trait_name is required for analysis.\n");
  if (covar_names_str == "all" && covar_file.empty())
    fail("\nError: --covariate_file is required when --covariate_names all is given.\n");
  if (covar_file.empty()) covar_file = phen_file;
  Inputs in;
  if (covar_names_str == "all") {
    CsvFile f = read_csv(covar_file);
    in.covar_names.assign(f.header.begin() + 1, f.header.end());
  } else if (!covar_names_str.empty()) {
    in.covar_names = split(covar_names_str, ',');
  }
  if (snp_info.empty()) fail("\nError: --snp_info_file is required for analysis.\n");
  if (bfile.empty()) fail("\nError: --binary_genotype_file is required for analysis.\n");
  if (min_maf < 0 || min_maf >= 0.5) fail("\nError: --min_maf is out of [0, 0.5).\n");
  if (min_hwep < 0 || min_hwep >= 1) fail("\nError: --min_hwe_pval is out of [0, 1).\n");
  if (out_file.empty()) fail("\nError: --output_file is required for analysis.\n");
  if (num_threads > 100 || num_threads < 1) fail("\nError: --num_threads is out of [1,100].\n");
  if (subset_size < 10 || subset_size > 5000) fail("\nError: --subset_size is out of [10, 5000].\n");
  if (num_rand < 3 || num_rand > 3000) fail("\nError: --num_rand_prob is out of [3, 3000].\n");
  if (num_qf < 3 || num_qf > 300) fail("\nError: --num_qf_markers is out of [3, 300].\n");
  if (!lmm && !using_ws) window_size = 20;
  if (window_size % 2 != 0) {
    std::cout << "\nWarning: --window_size is reset to its clostest even number.\n";
    window_size = window_size / 2 * 2;
  }
  if (lmm) {
    if (window_size < 10 || window_size > 5000) fail("\nError: --window_size is out of [10, 5000] for --lmm.\n");
  } else if (window_size < 0) {
    fail("\nError: --window_size is negative.\n");
  }
  if ((reml || lmm) && !snp_group.empty()) {
    std::cout << "\nWarning: --snp_set_name is temporarily disabled in --reml or --lmm.\n";
    snp_group.clear();
  }
  if (fake_geno) fail("\nError: --fake_geno is not supported by this build.\n");
  const int prec = precision_code(precision);

  // ---- inputs ----
  auto pheno = read_phenotypes(phen_file, trait, err_weight);
  auto covar = read_covariates(covar_file, in.covar_names);
  auto info = read_snp_info(snp_info, snp_group, snp_weight);
  if (!(file_exists(bfile + ".fam") && file_exists(bfile + ".bim") && file_exists(bfile + ".bed")))
    fail("\nError: bed/bim/fam fileset NOT found.\n");
  std::cout << "\nReading PLINK FAM file from [" + bfile + ".fam]." << std::endl;
  const std::vector<std::string> fam = read_fam(bfile + ".fam");
  in.n_fam = (int64_t)fam.size();
  for (size_t i = 0; i < fam.size(); ++i)
    if (pheno.count(fam[i]) && covar.count(fam[i])) {
      in.indi.push_back(fam[i]);
      in.keep_idx.push_back((int64_t)i);
    }
  if (in.indi.empty()) die("Individual set retained for analysis is empty.");
  const int64_t n = (int64_t)in.indi.size();
  const int c = (int)in.covar_names.size();
  std::cout << "Number of individuals retained in analysis = " << n << std::endl;
  in.y.resize(n);
  in.r.resize(n);
  in.X.resize((size_t)n * c);
  for (int64_t i = 0; i < n; ++i) {
    in.y[i] = pheno[in.indi[i]].first;
    in.r[i] = pheno[in.indi[i]].second;
    const std::vector<float>& v = covar[in.indi[i]];
    for (int j = 0; j < c; ++j) in.X[(size_t)j * n + i] = v[j];
  }
  std::cout << "\nReading PLINK BIM file from [" + bfile + ".bim]." << std::endl;
  in.bim = read_bim(bfile + ".bim");
  std::vector<int64_t> cand;   // .bim rows in the SNP info file
  for (size_t j = 0; j < in.bim.size(); ++j)
    if (info.count(in.bim[j].snp)) cand.push_back((int64_t)j);
  if (cand.empty()) die("Marker set for analysis is empty.");
  std::cout << "Size of marker set before MAF filtering = " << cand.size() << std::endl;
  std::cout << "\nReading PLINK BED file from [" + bfile + ".bed] in SNP-major format..." << std::endl;
  std::vector<uint8_t> rows = read_bed_rows(bfile + ".bed", in.n_fam, (int64_t)in.bim.size(), cand);
  const int64_t rb = (in.n_fam + 3) / 4;

  // ---- marker QC on the GPU (src/weight.cpp:3-15, src/input.cpp:10-22), filters, groups ----
  check(slemm_gpu_init(device));
  slemm_geno* G = nullptr;
  check(slemm_gpu_genotype_create(rows.data(), in.n_fam, (int64_t)cand.size(), rb, in.keep_idx.data(), n, 0, &G));
  std::vector<float> maf_c(cand.size()), hwe_c(cand.size());
  check(slemm_gpu_marker_qc(G, hwe_midp, maf_c.data(), hwe_c.data()));
  std::cout << "Calculating minor allele frequency..." << std::endl;
  int64_t low_maf = 0, low_hwe = 0;
  for (size_t q = 0; q < cand.size(); ++q) {
    low_maf += maf_c[q] <= min_maf;
    low_hwe += hwe_c[q] < min_hwep;
  }
  std::cout << low_maf << " markers of minor allele frequency <= " << min_maf << " are removed." << std::endl;
  std::cout << low_hwe << " markers fail in HWE tests: P<" << min_hwep << std::endl;
  Markers mk;
  std::map<std::string, std::vector<size_t>> by_group;   // candidate positions per group
  for (size_t q = 0; q < cand.size(); ++q) {
    if (!(maf_c[q] > min_maf && hwe_c[q] >= min_hwep)) continue;
    const std::string& s = in.bim[cand[q]].snp;
    by_group[info[s].first].push_back(q);
    mk.maf[s] = maf_c[q];
    mk.hwep[s] = hwe_c[q];
  }
  if (mk.maf.empty()) die("Marker set is empty.");
  if (beta_params.first != 1 && beta_params.second != 1) {
    std::cout << "\nWeighting markers for heritability using Beta PDF:\n";
    printf("Weight ~ X^(%.3f-1)*(1-X)^(%.3f-1), where X=MAF.\n\n", beta_params.first, beta_params.second);
    for (const auto& [s, f] : mk.maf) info[s].second = beta_pdf(beta_params.first, beta_params.second, f);
  }
  std::vector<size_t> order;
  for (const auto& [grp, qs] : by_group) {
    mk.group_order.push_back(grp);
    mk.group_size.push_back((int64_t)qs.size());
    for (size_t q : qs) {
      const std::string& s = in.bim[cand[q]].snp;
      mk.names.push_back(s);
      mk.groups.push_back(grp);
      mk.bim_idx.push_back(cand[q]);
      mk.weight.push_back(info[s].second);
      order.push_back(q);
    }
  }
  const int64_t m = (int64_t)mk.names.size();
  std::cout << "Number of markers retained = " << m << std::endl;
  std::cout << "Number of groups retained = " << mk.group_order.size() << std::endl;
  bool same = (int64_t)order.size() == (int64_t)cand.size();
  for (size_t k = 0; same && k < order.size(); ++k) same = order[k] == k;
  if (!same) {   // the analysis set differs from the candidates: pack its rows in its order
    std::vector<uint8_t> kept((size_t)m * rb);
    for (int64_t k = 0; k < m; ++k)
      std::copy(rows.begin() + order[k] * rb, rows.begin() + (order[k] + 1) * rb, kept.begin() + k * rb);
    slemm_gpu_genotype_destroy(G);
    G = nullptr;
    check(slemm_gpu_genotype_create(kept.data(), in.n_fam, m, rb, in.keep_idx.data(), n, 0, &G));
  }
  rows.clear();
  rows.shrink_to_fit();
  check(slemm_gpu_set_precision(G, prec));
  if (gpu_autotune) check(slemm_gpu_set_autotune(G, 1));
  if (gpu_reorth) check(slemm_gpu_set_lanczos(G, SLEMM_LANCZOS_REORTH));

  std::vector<float> Py(n, 0.f), snp_blup(m, 0.f), blue(c, 0.f), var_blue;
  float vg = 0, ve = 0, llr = 0;
  slemm_reml_opts o{num_rand, seed, rel_tol, max_h2, 1e-4f, 1e-4f, 600, 1};
  slemm_reml_result res{};
  const int n_mc = std::max(std::min(int(4e9 / n / n), 30), 3);
  int status = SLEMM_OK;
  if (wls) {
    status = slemm_gpu_wls(G, in.r.data(), in.X.data(), n, c, in.y.data(), snp_blup.data());
    if (status == SLEMM_OK) write_reml(out_file, in, mk, Py, snp_blup, blue, var_blue, vg, ve, llr);
  } else if (lmm) {
    if (m < window_size + 1) {
      slemm_gpu_genotype_destroy(G);
      fail("\nError: --window_size >= # of SNPs kept for --lmm.\n");
    }
    o.n_V = n_mc;
    status = slemm_gpu_reml_lmc(G, in.r.data(), in.X.data(), n, c, in.y.data(), mk.weight.data(), &o, Py.data(),
                                snp_blup.data(), blue.data(), &res);
    if (status == SLEMM_OK) {
      vg = res.vg;
      ve = res.ve;
      std::vector<int64_t> var(num_qf);
      std::vector<float> xPy(num_qf), xPx(num_qf), xBx(num_qf), xSx(num_qf);
      int cnt = 0;
      status = slemm_gpu_lmm_quadforms(G, Py.data(), ve / vg, rel_tol, num_qf, window_size, var.data(), xPy.data(),
                                       xPx.data(), xBx.data(), xSx.data(), &cnt);
      if (status == SLEMM_OK) {
        var.resize(cnt);
        write_reml(out_file, in, mk, Py, snp_blup, blue, var_blue, vg, ve, llr);
        write_gstat(out_file, in, mk, window_size, vg, var, xPy, xPx, xBx, xSx);
      }
    }
  } else {   // --reml
    std::vector<float> persnp = mk.weight;
    if (iter_weighting && m < window_size + 1) {
      std::cout << "\nWarning: --window_size >= total # of SNPs in --iter_weighting.\n";
      std::cout << "--iter_weighting is thus disabled.\n";
      iter_weighting = false;
    }
    if (!iter_weighting) {
      double s = 0;
      for (float w : persnp) s += w;
      const float mean = (float)(s / m);
      for (float& w : persnp) w /= mean;
      if (lrt) {
        var_blue.assign((size_t)c * c, 0.f);
        status = slemm_gpu_reml_sldf(G, in.r.data(), in.X.data(), n, c, in.y.data(), persnp.data(), &o, Py.data(),
                                     snp_blup.data(), blue.data(), var_blue.data(), &res);
        llr = res.lrt;
      } else {
        o.n_V = using_nr ? num_rand : n_mc;
        status = slemm_gpu_reml_lmc(G, in.r.data(), in.X.data(), n, c, in.y.data(), persnp.data(), &o, Py.data(),
                                    snp_blup.data(), blue.data(), &res);
      }
    } else {
      std::cout << "\nIterative SNP weighting with window size = " << window_size << "\n";
      const int max_fixed = SLEMM_MAX_COVARIATES - c;
      slemm_window_opts w{window_size, sig_chisq, indep_r2, lrt ? 1 : 0, n_mc, using_nr ? num_rand : 0, max_fixed};
      std::vector<float> blue_all((size_t)c + max_fixed), vb_all(lrt ? (size_t)SLEMM_MAX_COVARIATES * SLEMM_MAX_COVARIATES : 0);
      std::vector<int64_t> fixed(max_fixed);
      std::vector<float> maf_k(m);
      for (int64_t k = 0; k < m; ++k) maf_k[k] = mk.maf[mk.names[k]];
      int n_fixed = 0;
      status = slemm_gpu_reml_iter_weighting(G, in.r.data(), in.X.data(), n, c, in.y.data(), persnp.data(),
                                             maf_k.data(), &o, &w, Py.data(), snp_blup.data(), blue_all.data(),
                                             lrt ? vb_all.data() : nullptr, nullptr, fixed.data(), &n_fixed, &res);
      if (status == SLEMM_OK) {
        if (n_fixed == 0) std::cout << "\nNo SNPs will be fitted as fixed effects.\n";
        else {
          std::cout << "\nThe following SNPs will be fitted as fixed effects:\n";
          for (int i = 0; i < n_fixed; ++i) std::cout << mk.names[fixed[i]] << "\n";
        }
        std::copy(blue_all.begin(), blue_all.begin() + c, blue.begin());
        if (lrt) {   // the covariates' block of the (c + n_fixed)² var(BLUE)
          const int cc = c + n_fixed;
          var_blue.assign((size_t)c * c, 0.f);
          for (int j = 0; j < c; ++j)
            for (int i = 0; i < c; ++i) var_blue[(size_t)j * c + i] = vb_all[(size_t)j * cc + i];
        }
        llr = lrt ? res.lrt : 0.f;
      }
    }
    if (status == SLEMM_OK) {
      vg = res.vg;
      ve = res.ve;
      write_reml(out_file, in, mk, Py, snp_blup, blue, var_blue, vg, ve, llr);
    }
  }
  slemm_gpu_genotype_destroy(G);
  check(status);
}

}  // namespace

int main(int argc, char** argv)
{
  std::cout << "*******************************************************************" << std::endl;
  std::cout << "* SLEMM on GB300 (libslemm_gb300)" << std::endl;
  std::cout << "* Stochastic-Lanczos-Expedited Mixed Models" << std::endl;
  std::cout << "*******************************************************************" << std::endl;
  const auto start = std::chrono::system_clock::now();
  const std::time_t t0 = std::chrono::system_clock::to_time_t(start);
  std::cout << "Analysis started: " << std::ctime(&t0) << std::endl;
  try {
    run(argc, argv);
  } catch (const Failure& f) {
    std::cerr << "\n" << f.msg << std::endl;
  } catch (const std::exception& e) {   // std::stof and friends on a malformed number
    std::cerr << "\nError: " << e.what() << std::endl;
  }
  const auto end = std::chrono::system_clock::now();
  const std::time_t t1 = std::chrono::system_clock::to_time_t(end);
  std::cout << "\nAnalysis finished: " << std::ctime(&t1);
  const long used = (long)std::chrono::duration<double>(end - start).count();
  std::cout << "Computational time: " << used / 3600 << ":" << (used % 3600) / 60 << ":" << used % 60 << std::endl;
  return 0;
}
