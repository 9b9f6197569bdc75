// parm7 topology reader/writer and Amber ASCII restart I/O.
//
// Replaces src/sff/prm.c:584 (rdparm), prm.c:1997 (wrparm), prm.c:2810
// (free_prm) and src/sff/sff.c:651/733 (getxv/putxv).  The reader produces
// the same PARMSTRUCT_T contents the reference does, which the energy code
// depends on:
//   - numbers are read as a whitespace-separated stream per section (the
//     reference uses fscanf " %lf"), names as fixed 4-character fields;
//   - new-format files are located by %FLAG name; old-format files are read
//     sequentially in the historical section order;
//   - RESIDUE_POINTER becomes 0-based with Ipres[Nres] = Natom (prm.c:900);
//   - SCEE/SCNB scale factors are stored inverted, default 1/1.2 and 1/2.0
//     when absent or in old-format files (prm.c:1070-1147);
//   - ATOMIC_NUMBER falls back to a mass lookup (prm.c:85, prm.c:1122);
//   - Fsmax = max Fs*(Rborn-0.09) (prm.c:1652-1656); old-format files get
//     Bondi radii and Tinker screening factors from the atom names
//     (prm.c:1664-1738);
//   - the 1-4 list is built from the dihedrals whose third and fourth atom
//     indices are non-negative, keyed on the smaller end atom
//     (prm.c:1855-1900).
#include "sffg_internal.h"

#include <cctype>
#include <cmath>
#include <cstdarg>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

namespace {

[[noreturn]] void prm_fail(const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  std::vfprintf(stderr, fmt, ap);
  va_end(ap);
  std::fputc('\n', stderr);
  std::exit(1);
}

template <class T> T *alloc_n(size_t n) {
  size_t bytes = (n ? n : 1) * sizeof(T);
  T *p = static_cast<T *>(std::calloc(1, bytes));
  if (!p) prm_fail("rdparm: out of memory (%zu bytes)", bytes);
  return p;
}

// Cursor over the lines of one section (new format) or of the whole file
// (old format).  Numeric reads consume whitespace-separated tokens across
// lines; after a numeric block the reader moves to the start of the next
// line, as the reference's skipeoln() does.
class LineCursor {
 public:
  explicit LineCursor(std::vector<std::string> lines) : lines_(std::move(lines)) {}

  bool next_token(std::string &tok) {
    while (line_ < lines_.size()) {
      const std::string &s = lines_[line_];
      while (col_ < s.size() && std::isspace(static_cast<unsigned char>(s[col_]))) col_++;
      if (col_ < s.size()) {
        size_t b = col_;
        while (col_ < s.size() && !std::isspace(static_cast<unsigned char>(s[col_]))) col_++;
        tok.assign(s, b, col_ - b);
        mid_line_ = true;
        return true;
      }
      line_++;
      col_ = 0;
      mid_line_ = false;
    }
    return false;
  }
  // Consume through the end of the current line, like the reference's
  // skipeoln(): the rest of the line after the last number read, or a whole
  // (typically blank) line when the block held no numbers.
  void end_numeric_block() {
    line_++;
    col_ = 0;
    mid_line_ = false;
  }
  bool next_line(std::string &s) {
    if (line_ >= lines_.size()) return false;
    s = lines_[line_].substr(col_);
    line_++;
    col_ = 0;
    mid_line_ = false;
    return true;
  }

 private:
  std::vector<std::string> lines_;
  size_t line_ = 0, col_ = 0;
  bool mid_line_ = false;
};

struct ParmSource {
  bool newparm = false;
  std::map<std::string, std::vector<std::string>> sections;  // new format
  LineCursor *seq = nullptr;                                  // old format
  std::string fname;
  LineCursor section_cursor_storage{{}};

  // Returns the cursor for a section, or nullptr when a new-format file
  // lacks it (optional sections only).
  LineCursor *open(const char *flag, bool required = true) {
    if (!newparm) return seq;
    auto it = sections.find(flag);
    if (it == sections.end()) {
      if (required) prm_fail("rdparm: %s: section %%FLAG %s not found", fname.c_str(), flag);
      return nullptr;
    }
    section_cursor_storage = LineCursor(it->second);
    return &section_cursor_storage;
  }
};

template <class T> void read_numbers(LineCursor *c, const char *what, T *dst, long n) {
  std::string tok;
  for (long i = 0; i < n; i++) {
    if (!c->next_token(tok)) prm_fail("rdparm: premature end of data in %s", what);
    char *end = nullptr;
    if constexpr (std::is_integral<T>::value) {
      dst[i] = static_cast<T>(std::strtol(tok.c_str(), &end, 10));
    } else {
      // Fortran D exponents are read like E exponents.
      for (char &ch : tok)
        if (ch == 'D' || ch == 'd') ch = 'E';
      dst[i] = static_cast<T>(std::strtod(tok.c_str(), &end));
    }
    if (end == tok.c_str()) prm_fail("rdparm: bad number '%s' in %s", tok.c_str(), what);
  }
  c->end_numeric_block();
}

void read_names(LineCursor *c, const char *what, NAME_T *dst, long n) {
  std::string line;
  for (long i = 0; i < n; i += 20) {
    if (!c->next_line(line)) prm_fail("rdparm: premature end of data in %s", what);
    for (long j = 0; j < 20 && i + j < n; j++) {
      std::memset(dst[i + j], ' ', 5);
      dst[i + j][5] = '\0';
      for (int k = 0; k < 4; k++) {
        size_t pos = static_cast<size_t>(4 * j + k);
        dst[i + j][k] = pos < line.size() ? line[pos] : ' ';
      }
    }
  }
}

// Element from mass, used when ATOMIC_NUMBER is absent (prm.c:85).
int atomic_number_from_mass(double m) {
  struct { double lo, hi; int z; } tab[] = {
      {0.9, 1.1, 1},    {3.9, 4.1, 2},    {6.9, 7.1, 3},    {8.9, 9.1, 4},
      {10.8, 10.9, 5},  {12.0, 12.1, 6},  {14.0, 14.1, 7},  {15.9, 16.1, 8},
      {18.9, 19.1, 9},  {20.1, 20.3, 10}, {22.9, 23.1, 11}, {24.2, 24.4, 12},
      {26.9, 27.1, 13}, {28.0, 28.2, 14}, {30.9, 31.1, 15}, {32.0, 32.2, 16},
      {35.4, 35.5, 17}, {39.0, 39.2, 19}, {39.9, 40.0, 18}, {40.0, 40.2, 20},
      {54.9, 55.0, 25}, {55.8, 55.9, 26}, {58.9, 59.0, 27}, {58.6, 58.8, 28},
      {63.5, 63.6, 29}, {65.3, 65.5, 30}, {79.9, 80.0, 35}, {126.9, 127.0, 53},
      {132.9, 133.0, 55},
  };
  for (auto &t : tab)
    if (m > t.lo && m < t.hi) return t.z;
  return 0;
}

void split_lines(const std::string &text, std::vector<std::string> &out) {
  size_t b = 0;
  while (b <= text.size()) {
    size_t e = text.find('\n', b);
    if (e == std::string::npos) e = text.size();
    std::string s = text.substr(b, e - b);
    if (!s.empty() && s.back() == '\r') s.pop_back();
    out.push_back(std::move(s));
    if (e == text.size()) break;
    b = e + 1;
  }
}

}  // namespace

namespace sffg {

void prm_finish_derived(PARMSTRUCT_T *prm, bool newparm) {
  // Fsmax with the historical fixed offset (prm.c:1652-1656).
  const double boffset = 0.09;
  prm->Fsmax = 0.0;
  for (int i = 0; i < prm->Natom; i++) {
    double s = prm->Fs[i] * (prm->Rborn[i] - boffset);
    if (s > prm->Fsmax) prm->Fsmax = s;
  }
  (void)newparm;
  // 1-4 list keyed on the smaller end atom (prm.c:1855-1900).
  const int maxper = 12;
  std::vector<int> partner(static_cast<size_t>(maxper) * prm->Natom);
  std::vector<int> dtype(static_cast<size_t>(maxper) * prm->Natom);
  for (int i = 0; i < prm->Natom; i++) prm->N14pairs[i] = 0;
  auto add_list = [&](int n, const int *a1, const int *a3, const int *a4, const int *num) {
    for (int i = 0; i < n; i++) {
      int iat = a1[i] / 3, kat = a3[i] / 3, lat = a4[i] / 3;
      if (kat >= 0 && lat >= 0) {
        int small = iat < lat ? iat : lat;
        int big = iat > lat ? iat : lat;
        int &cnt = prm->N14pairs[small];
        if (cnt >= maxper) prm_fail("rdparm: atom %d has more than %d 1-4 partners", small + 1, maxper);
        partner[static_cast<size_t>(maxper) * small + cnt] = big;
        dtype[static_cast<size_t>(maxper) * small + cnt] = num[i] - 1;
        cnt++;
      }
    }
  };
  add_list(prm->Nphih, prm->DihHAt1, prm->DihHAt3, prm->DihHAt4, prm->DihHNum);
  add_list(prm->Mphia, prm->DihAt1, prm->DihAt3, prm->DihAt4, prm->DihNum);
  int total = 0;
  for (int i = 0; i < prm->Natom; i++) total += prm->N14pairs[i];
  std::free(prm->N14pairlist);
  std::free(prm->N14sceelist);
  std::free(prm->N14scnblist);
  prm->N14pairlist = alloc_n<int>(total);
  prm->N14sceelist = alloc_n<double>(total);
  prm->N14scnblist = alloc_n<double>(total);
  int k = 0;
  for (int i = 0; i < prm->Natom - 1; i++) {
    for (int m = 0; m < prm->N14pairs[i]; m++) {
      size_t s = static_cast<size_t>(maxper) * i + m;
      prm->N14pairlist[k] = partner[s];
      prm->N14sceelist[k] = prm->Scee[dtype[s]];
      prm->N14scnblist[k] = prm->Scnb[dtype[s]];
      k++;
    }
  }
}

void prm_allocate_arrays(PARMSTRUCT_T *prm) {
  prm->Nat3 = 3 * prm->Natom;
  prm->Ntype2d = prm->Ntypes * prm->Ntypes;
  prm->Nttyp = prm->Ntypes * (prm->Ntypes + 1) / 2;
  const int na = prm->Natom;
  prm->AtomNames = alloc_n<NAME_T>(na);
  prm->Charges = alloc_n<double>(na);
  prm->Masses = alloc_n<double>(na);
  prm->Iac = alloc_n<int>(na);
  prm->Iblo = alloc_n<int>(na);
  prm->Cno = alloc_n<int>(prm->Ntype2d);
  prm->ResNames = alloc_n<NAME_T>(prm->Nres + 1);
  prm->Ipres = alloc_n<int>(prm->Nres + 1);
  prm->Rk = alloc_n<double>(prm->Numbnd);
  prm->Req = alloc_n<double>(prm->Numbnd);
  prm->Tk = alloc_n<double>(prm->Numang);
  prm->Teq = alloc_n<double>(prm->Numang);
  prm->Pk = alloc_n<double>(prm->Nptra);
  prm->Pn = alloc_n<double>(prm->Nptra);
  prm->Phase = alloc_n<double>(prm->Nptra);
  prm->Scee = alloc_n<double>(prm->Nptra);
  prm->Scnb = alloc_n<double>(prm->Nptra);
  prm->Solty = alloc_n<double>(prm->Natyp);
  prm->Cn1 = alloc_n<double>(prm->Nttyp);
  prm->Cn2 = alloc_n<double>(prm->Nttyp);
  prm->BondHAt1 = alloc_n<int>(prm->Nbonh);
  prm->BondHAt2 = alloc_n<int>(prm->Nbonh);
  prm->BondHNum = alloc_n<int>(prm->Nbonh);
  prm->BondAt1 = alloc_n<int>(prm->Nbona);
  prm->BondAt2 = alloc_n<int>(prm->Nbona);
  prm->BondNum = alloc_n<int>(prm->Nbona);
  prm->AngleHAt1 = alloc_n<int>(prm->Ntheth);
  prm->AngleHAt2 = alloc_n<int>(prm->Ntheth);
  prm->AngleHAt3 = alloc_n<int>(prm->Ntheth);
  prm->AngleHNum = alloc_n<int>(prm->Ntheth);
  prm->AngleAt1 = alloc_n<int>(prm->Ntheta);
  prm->AngleAt2 = alloc_n<int>(prm->Ntheta);
  prm->AngleAt3 = alloc_n<int>(prm->Ntheta);
  prm->AngleNum = alloc_n<int>(prm->Ntheta);
  prm->DihHAt1 = alloc_n<int>(prm->Nphih);
  prm->DihHAt2 = alloc_n<int>(prm->Nphih);
  prm->DihHAt3 = alloc_n<int>(prm->Nphih);
  prm->DihHAt4 = alloc_n<int>(prm->Nphih);
  prm->DihHNum = alloc_n<int>(prm->Nphih);
  prm->DihAt1 = alloc_n<int>(prm->Nphia);
  prm->DihAt2 = alloc_n<int>(prm->Nphia);
  prm->DihAt3 = alloc_n<int>(prm->Nphia);
  prm->DihAt4 = alloc_n<int>(prm->Nphia);
  prm->DihNum = alloc_n<int>(prm->Nphia);
  prm->ExclAt = alloc_n<int>(prm->Nnb);
  prm->HB12 = alloc_n<double>(prm->Nphb);
  prm->HB10 = alloc_n<double>(prm->Nphb);
  prm->AtomType = alloc_n<NAME_T>(na);
  prm->AtomTree = alloc_n<NAME_T>(na);
  prm->TreeJoin = alloc_n<int>(na);
  prm->AtomRes = alloc_n<int>(na);
  prm->Rborn = alloc_n<double>(na);
  prm->Fs = alloc_n<double>(na);
  prm->Gvdw = alloc_n<double>(na);
  prm->AtomicNum = alloc_n<int>(na);
  prm->N14pairs = alloc_n<int>(na);
  prm->N14pairlist = nullptr;
  prm->N14sceelist = nullptr;
  prm->N14scnblist = nullptr;
  prm->Nspm = 1;
  prm->Boundary = alloc_n<int>(1);
  prm->Boundary[0] = na;
  prm->Box[0] = prm->Box[1] = prm->Box[2] = 999999999.;
  prm->Nstrand = prm->Ncomplex = 1;
  prm->Ipstrand = alloc_n<int>(2);
  prm->Ipcomplex = alloc_n<int>(2);
}

}  // namespace sffg

extern "C" PARMSTRUCT_T *rdparm(STRING_T *name) {
  std::ifstream in(name, std::ios::binary);
  if (!in) prm_fail("Cannot read parm file %s", name);
  std::stringstream ss;
  ss << in.rdbuf();
  std::vector<std::string> lines;
  split_lines(ss.str(), lines);
  if (sffg::legacy_out()) std::fprintf(sffg::legacy_out(), "Reading parm file (%s)\n", name);

  ParmSource src;
  src.fname = name;
  PARMSTRUCT_T *prm = alloc_n<PARMSTRUCT_T>(1);
  LineCursor whole(lines);
  std::string title;
  if (!lines.empty() && lines[0].compare(0, 8, "%VERSION") == 0) {
    src.newparm = true;
    std::string cur;
    for (size_t i = 0; i < lines.size(); i++) {
      const std::string &s = lines[i];
      if (s.compare(0, 5, "%FLAG") == 0) {
        size_t b = 5;
        while (b < s.size() && s[b] == ' ') b++;
        size_t e = b;
        while (e < s.size() && s[e] != ' ') e++;
        cur = s.substr(b, e - b);
        src.sections[cur];
        if (i + 1 < lines.size() && lines[i + 1].compare(0, 7, "%FORMAT") == 0) i++;
      } else if (!cur.empty() && s.compare(0, 8, "%COMMENT") != 0) {
        src.sections[cur].push_back(s);
      }
    }
    auto it = src.sections.find("TITLE");
    if (it != src.sections.end() && !it->second.empty()) title = it->second[0];
  } else {
    src.seq = &whole;
    whole.next_line(title);
  }
  std::strncpy(prm->ititl, title.c_str(), 80);
  prm->ititl[80] = '\0';
  if (sffg::legacy_out()) std::fprintf(sffg::legacy_out(), "title:\n%s\n", prm->ititl);

  LineCursor *c = src.open("POINTERS");
  int ptr[31] = {0};
  read_numbers(c, "POINTERS", ptr, 30);
  prm->Natom = ptr[0];  prm->Ntypes = ptr[1]; prm->Nbonh = ptr[2];  prm->Mbona = ptr[3];
  prm->Ntheth = ptr[4]; prm->Mtheta = ptr[5]; prm->Nphih = ptr[6];  prm->Mphia = ptr[7];
  prm->Nhparm = ptr[8]; prm->Nparm = ptr[9];  prm->Nnb = ptr[10];   prm->Nres = ptr[11];
  prm->Nbona = ptr[12]; prm->Ntheta = ptr[13]; prm->Nphia = ptr[14]; prm->Numbnd = ptr[15];
  prm->Numang = ptr[16]; prm->Nptra = ptr[17]; prm->Natyp = ptr[18]; prm->Nphb = ptr[19];
  prm->IfBox = ptr[27]; prm->Nmxrs = ptr[28]; prm->IfCap = ptr[29];
  if (src.newparm) {
    // An optional 31st pointer (NUMEXTRA) may follow on the same section.
    std::string tok;
    prm->Numextra = c->next_token(tok) ? std::atoi(tok.c_str()) : 0;
  }
  if (prm->Natom <= 0) prm_fail("rdparm: %s: bad atom count %d", name, prm->Natom);
  if (prm->IfBox) {
    if (sffg::legacy_out()) std::fprintf(sffg::legacy_out(), "periodic prmtop found, not supported by NAB\n");
    std::exit(1);
  }
  sffg::prm_allocate_arrays(prm);

  read_names(src.open("ATOM_NAME"), "ATOM_NAME", prm->AtomNames, prm->Natom);
  read_numbers(src.open("CHARGE"), "CHARGE", prm->Charges, prm->Natom);
  read_numbers(src.open("MASS"), "MASS", prm->Masses, prm->Natom);
  read_numbers(src.open("ATOM_TYPE_INDEX"), "ATOM_TYPE_INDEX", prm->Iac, prm->Natom);
  read_numbers(src.open("NUMBER_EXCLUDED_ATOMS"), "NUMBER_EXCLUDED_ATOMS", prm->Iblo, prm->Natom);
  read_numbers(src.open("NONBONDED_PARM_INDEX"), "NONBONDED_PARM_INDEX", prm->Cno, prm->Ntype2d);
  read_names(src.open("RESIDUE_LABEL"), "RESIDUE_LABEL", prm->ResNames, prm->Nres);
  read_numbers(src.open("RESIDUE_POINTER"), "RESIDUE_POINTER", prm->Ipres, prm->Nres);
  for (int i = 0; i < prm->Nres; i++) prm->Ipres[i] -= 1;
  prm->Ipres[prm->Nres] = prm->Natom;
  read_numbers(src.open("BOND_FORCE_CONSTANT"), "BOND_FORCE_CONSTANT", prm->Rk, prm->Numbnd);
  read_numbers(src.open("BOND_EQUIL_VALUE"), "BOND_EQUIL_VALUE", prm->Req, prm->Numbnd);
  read_numbers(src.open("ANGLE_FORCE_CONSTANT"), "ANGLE_FORCE_CONSTANT", prm->Tk, prm->Numang);
  read_numbers(src.open("ANGLE_EQUIL_VALUE"), "ANGLE_EQUIL_VALUE", prm->Teq, prm->Numang);
  read_numbers(src.open("DIHEDRAL_FORCE_CONSTANT"), "DIHEDRAL_FORCE_CONSTANT", prm->Pk, prm->Nptra);
  read_numbers(src.open("DIHEDRAL_PERIODICITY"), "DIHEDRAL_PERIODICITY", prm->Pn, prm->Nptra);
  for (int i = 0; i < prm->Nptra; i++)
    if (prm->Pn[i] == 0) prm_fail("Found an invalid periodicity in the prmtop file: %d", i);
  read_numbers(src.open("DIHEDRAL_PHASE"), "DIHEDRAL_PHASE", prm->Phase, prm->Nptra);
  for (int i = 0; i < prm->Nptra; i++) {
    prm->Scee[i] = 1.0 / 1.2;
    prm->Scnb[i] = 1.0 / 2.0;
  }
  if (src.newparm) {
    if (LineCursor *s = src.open("SCEE_SCALE_FACTOR", false)) {
      read_numbers(s, "SCEE_SCALE_FACTOR", prm->Scee, prm->Nptra);
      for (int i = 0; i < prm->Nptra; i++) prm->Scee[i] = 1.0 / prm->Scee[i];
    }
    if (LineCursor *s = src.open("SCNB_SCALE_FACTOR", false)) {
      read_numbers(s, "SCNB_SCALE_FACTOR", prm->Scnb, prm->Nptra);
      for (int i = 0; i < prm->Nptra; i++) prm->Scnb[i] = 1.0 / prm->Scnb[i];
    }
    if (LineCursor *s = src.open("ATOMIC_NUMBER", false)) {
      read_numbers(s, "ATOMIC_NUMBER", prm->AtomicNum, prm->Natom);
    } else {
      for (int i = 0; i < prm->Natom; i++) prm->AtomicNum[i] = atomic_number_from_mass(prm->Masses[i]);
    }
  }
  read_numbers(src.open("SOLTY"), "SOLTY", prm->Solty, prm->Natyp);
  read_numbers(src.open("LENNARD_JONES_ACOEF"), "LENNARD_JONES_ACOEF", prm->Cn1, prm->Nttyp);
  read_numbers(src.open("LENNARD_JONES_BCOEF"), "LENNARD_JONES_BCOEF", prm->Cn2, prm->Nttyp);
  {
    std::vector<int> t(3 * static_cast<size_t>(prm->Nbonh));
    read_numbers(src.open("BONDS_INC_HYDROGEN"), "BONDS_INC_HYDROGEN", t.data(), 3L * prm->Nbonh);
    for (int i = 0; i < prm->Nbonh; i++) {
      prm->BondHAt1[i] = t[3 * i]; prm->BondHAt2[i] = t[3 * i + 1]; prm->BondHNum[i] = t[3 * i + 2];
    }
  }
  {
    std::vector<int> t(3 * static_cast<size_t>(prm->Nbona));
    read_numbers(src.open("BONDS_WITHOUT_HYDROGEN"), "BONDS_WITHOUT_HYDROGEN", t.data(), 3L * prm->Nbona);
    for (int i = 0; i < prm->Nbona; i++) {
      prm->BondAt1[i] = t[3 * i]; prm->BondAt2[i] = t[3 * i + 1]; prm->BondNum[i] = t[3 * i + 2];
    }
  }
  {
    std::vector<int> t(4 * static_cast<size_t>(prm->Ntheth));
    read_numbers(src.open("ANGLES_INC_HYDROGEN"), "ANGLES_INC_HYDROGEN", t.data(), 4L * prm->Ntheth);
    for (int i = 0; i < prm->Ntheth; i++) {
      prm->AngleHAt1[i] = t[4 * i]; prm->AngleHAt2[i] = t[4 * i + 1];
      prm->AngleHAt3[i] = t[4 * i + 2]; prm->AngleHNum[i] = t[4 * i + 3];
    }
  }
  {
    std::vector<int> t(4 * static_cast<size_t>(prm->Ntheta));
    read_numbers(src.open("ANGLES_WITHOUT_HYDROGEN"), "ANGLES_WITHOUT_HYDROGEN", t.data(), 4L * prm->Ntheta);
    for (int i = 0; i < prm->Ntheta; i++) {
      prm->AngleAt1[i] = t[4 * i]; prm->AngleAt2[i] = t[4 * i + 1];
      prm->AngleAt3[i] = t[4 * i + 2]; prm->AngleNum[i] = t[4 * i + 3];
    }
  }
  {
    std::vector<int> t(5 * static_cast<size_t>(prm->Nphih));
    read_numbers(src.open("DIHEDRALS_INC_HYDROGEN"), "DIHEDRALS_INC_HYDROGEN", t.data(), 5L * prm->Nphih);
    for (int i = 0; i < prm->Nphih; i++) {
      prm->DihHAt1[i] = t[5 * i]; prm->DihHAt2[i] = t[5 * i + 1]; prm->DihHAt3[i] = t[5 * i + 2];
      prm->DihHAt4[i] = t[5 * i + 3]; prm->DihHNum[i] = t[5 * i + 4];
    }
  }
  {
    std::vector<int> t(5 * static_cast<size_t>(prm->Nphia));
    read_numbers(src.open("DIHEDRALS_WITHOUT_HYDROGEN"), "DIHEDRALS_WITHOUT_HYDROGEN", t.data(), 5L * prm->Nphia);
    for (int i = 0; i < prm->Nphia; i++) {
      prm->DihAt1[i] = t[5 * i]; prm->DihAt2[i] = t[5 * i + 1]; prm->DihAt3[i] = t[5 * i + 2];
      prm->DihAt4[i] = t[5 * i + 3]; prm->DihNum[i] = t[5 * i + 4];
    }
  }
  read_numbers(src.open("EXCLUDED_ATOMS_LIST"), "EXCLUDED_ATOMS_LIST", prm->ExclAt, prm->Nnb);
  read_numbers(src.open("HBOND_ACOEF"), "HBOND_ACOEF", prm->HB12, prm->Nphb);
  read_numbers(src.open("HBOND_BCOEF"), "HBOND_BCOEF", prm->HB10, prm->Nphb);
  {
    std::vector<double> hbcut(prm->Nphb + 1);
    read_numbers(src.open("HBCUT"), "HBCUT", hbcut.data(), prm->Nphb);
  }
  read_names(src.open("AMBER_ATOM_TYPE"), "AMBER_ATOM_TYPE", prm->AtomType, prm->Natom);
  read_names(src.open("TREE_CHAIN_CLASSIFICATION"), "TREE_CHAIN_CLASSIFICATION", prm->AtomTree, prm->Natom);
  read_numbers(src.open("JOIN_ARRAY"), "JOIN_ARRAY", prm->TreeJoin, prm->Natom);
  read_numbers(src.open("IROTAT"), "IROTAT", prm->AtomRes, prm->Natom);
  for (int i = 0, res = 0; i < prm->Natom; i++) {
    if (res + 1 <= prm->Nres && i == prm->Ipres[res + 1]) res++;
    prm->AtomRes[i] = res;
  }

  if (src.newparm) {
    read_numbers(src.open("RADII"), "RADII", prm->Rborn, prm->Natom);
    read_numbers(src.open("SCREEN"), "SCREEN", prm->Fs, prm->Natom);
  } else {
    // Bondi radii / Tinker screening factors from the first letter of the
    // atom name, for old-format files (prm.c:1664-1738).
    if (sffg::legacy_out())
      std::fprintf(sffg::legacy_out(), "old prmtop format => using old algorithm for GB parms\n");
    for (int i = 0; i < prm->Natom; i++) {
      char a = prm->AtomNames[i][0];
      switch (a) {
        case 'H': {
          char p = 'O';
          if (i > 0) {
            for (int j = 1; j <= 3; j++) {
              p = prm->AtomNames[i - j][0];
              if (p != 'H') break;
            }
          }
          prm->Fs[i] = 0.85;
          prm->Rborn[i] = p == 'O' ? 0.8 : p == 'N' ? 1.2 : p == 'C' ? 1.3 : 1.2;
          break;
        }
        case 'C': prm->Fs[i] = 0.72; prm->Rborn[i] = 1.70; break;
        case 'N': prm->Fs[i] = 0.79; prm->Rborn[i] = 1.55; break;
        case 'O': prm->Fs[i] = 0.85; prm->Rborn[i] = 1.50; break;
        case 'F': prm->Fs[i] = 0.88; prm->Rborn[i] = 1.47; break;
        case 'P': prm->Fs[i] = 0.86; prm->Rborn[i] = 1.85; break;
        case 'S': prm->Fs[i] = 0.96; prm->Rborn[i] = 1.80; break;
        case 'L': prm->Fs[i] = 0.96; prm->Rborn[i] = 1.00; break;
        case 'Z': prm->Fs[i] = 0.96; prm->Rborn[i] = 1.40; break;
        case 'M': prm->Fs[i] = 0.96; prm->Rborn[i] = 1.40; break;
        default: prm_fail("bad atom symbol: %d, %c", i, a);
      }
    }
  }
  sffg::prm_finish_derived(prm, src.newparm);
  return prm;
}

extern "C" INT_T free_prm(PARMSTRUCT_T *prm) {
  if (!prm) return 0;
  void *ptrs[] = {
      prm->AtomNames, prm->ResNames, prm->AtomType, prm->AtomTree, prm->Charges, prm->Masses,
      prm->Rk, prm->Req, prm->Tk, prm->Teq, prm->Pk, prm->Pn, prm->Phase, prm->Solty, prm->Cn1,
      prm->Cn2, prm->HB12, prm->HB10, prm->Rborn, prm->Fs, prm->Iac, prm->Iblo, prm->Cno,
      prm->Ipres, prm->ExclAt, prm->TreeJoin, prm->AtomRes, prm->BondHAt1, prm->BondHAt2,
      prm->BondHNum, prm->BondAt1, prm->BondAt2, prm->BondNum, prm->AngleHAt1, prm->AngleHAt2,
      prm->AngleHAt3, prm->AngleHNum, prm->AngleAt1, prm->AngleAt2, prm->AngleAt3, prm->AngleNum,
      prm->DihHAt1, prm->DihHAt2, prm->DihHAt3, prm->DihHAt4, prm->DihHNum, prm->DihAt1,
      prm->DihAt2, prm->DihAt3, prm->DihAt4, prm->DihNum, prm->Boundary, prm->AtomicNum,
      prm->N14pairs, prm->N14pairlist, prm->Gvdw, prm->Scee, prm->Scnb, prm->N14sceelist,
      prm->N14scnblist, prm->Ipstrand, prm->Ipcomplex};
  for (void *p : ptrs) std::free(p);
  std::free(prm);
  return 0;
}

namespace {

void write_section(FILE *fp, const char *flag, const char *fmt) {
  std::fprintf(fp, "%%FLAG %-74s\n%%FORMAT(%s)\n", flag, fmt);
}

template <class F> void write_block(FILE *fp, long n, int per_line, F emit) {
  if (n == 0) {
    std::fputc('\n', fp);
    return;
  }
  for (long i = 0; i < n; i++) {
    emit(i);
    if ((i + 1) % per_line == 0 || i + 1 == n) std::fputc('\n', fp);
  }
}

void write_ints(FILE *fp, const char *flag, const int *v, long n) {
  write_section(fp, flag, "10I8");
  write_block(fp, n, 10, [&](long i) { std::fprintf(fp, "%8d", v[i]); });
}

void write_reals(FILE *fp, const char *flag, const double *v, long n) {
  write_section(fp, flag, "5E16.8");
  write_block(fp, n, 5, [&](long i) { std::fprintf(fp, "%16.8E", v[i]); });
}

void write_names(FILE *fp, const char *flag, const NAME_T *v, long n) {
  write_section(fp, flag, "20a4");
  write_block(fp, n, 20, [&](long i) { std::fprintf(fp, "%-4.4s", v[i]); });
}

}  // namespace

extern "C" INT_T wrparm(PARMSTRUCT_T *prm, STRING_T *name) {
  FILE *fp = std::fopen(name, "w");
  if (!fp) return -1;
  std::fprintf(fp, "%%VERSION  VERSION_STAMP = V0001.000  DATE = 01/01/26  00:00:00\n");
  write_section(fp, "TITLE", "20a4");
  std::fprintf(fp, "%-80.80s\n", prm->ititl);
  int ptr[31] = {prm->Natom, prm->Ntypes, prm->Nbonh, prm->Mbona, prm->Ntheth, prm->Mtheta,
                 prm->Nphih, prm->Mphia, prm->Nhparm, prm->Nparm, prm->Nnb, prm->Nres,
                 prm->Nbona, prm->Ntheta, prm->Nphia, prm->Numbnd, prm->Numang, prm->Nptra,
                 prm->Natyp, prm->Nphb, 0, 0, 0, 0, 0, 0, 0, prm->IfBox, prm->Nmxrs,
                 prm->IfCap, 0};
  write_ints(fp, "POINTERS", ptr, 31);
  write_names(fp, "ATOM_NAME", prm->AtomNames, prm->Natom);
  write_reals(fp, "CHARGE", prm->Charges, prm->Natom);
  write_ints(fp, "ATOMIC_NUMBER", prm->AtomicNum, prm->Natom);
  write_reals(fp, "MASS", prm->Masses, prm->Natom);
  write_ints(fp, "ATOM_TYPE_INDEX", prm->Iac, prm->Natom);
  write_ints(fp, "NUMBER_EXCLUDED_ATOMS", prm->Iblo, prm->Natom);
  write_ints(fp, "NONBONDED_PARM_INDEX", prm->Cno, prm->Ntype2d);
  write_names(fp, "RESIDUE_LABEL", prm->ResNames, prm->Nres);
  {
    std::vector<int> ip(prm->Nres);
    for (int i = 0; i < prm->Nres; i++) ip[i] = prm->Ipres[i] + 1;
    write_ints(fp, "RESIDUE_POINTER", ip.data(), prm->Nres);
  }
  write_reals(fp, "BOND_FORCE_CONSTANT", prm->Rk, prm->Numbnd);
  write_reals(fp, "BOND_EQUIL_VALUE", prm->Req, prm->Numbnd);
  write_reals(fp, "ANGLE_FORCE_CONSTANT", prm->Tk, prm->Numang);
  write_reals(fp, "ANGLE_EQUIL_VALUE", prm->Teq, prm->Numang);
  write_reals(fp, "DIHEDRAL_FORCE_CONSTANT", prm->Pk, prm->Nptra);
  write_reals(fp, "DIHEDRAL_PERIODICITY", prm->Pn, prm->Nptra);
  write_reals(fp, "DIHEDRAL_PHASE", prm->Phase, prm->Nptra);
  {
    std::vector<double> s(prm->Nptra);
    for (int i = 0; i < prm->Nptra; i++) s[i] = 1.0 / prm->Scee[i];
    write_reals(fp, "SCEE_SCALE_FACTOR", s.data(), prm->Nptra);
    for (int i = 0; i < prm->Nptra; i++) s[i] = 1.0 / prm->Scnb[i];
    write_reals(fp, "SCNB_SCALE_FACTOR", s.data(), prm->Nptra);
  }
  write_reals(fp, "SOLTY", prm->Solty, prm->Natyp);
  write_reals(fp, "LENNARD_JONES_ACOEF", prm->Cn1, prm->Nttyp);
  write_reals(fp, "LENNARD_JONES_BCOEF", prm->Cn2, prm->Nttyp);
  auto interleave = [](std::vector<int> &out, std::initializer_list<const int *> cols, int n) {
    out.clear();
    for (int i = 0; i < n; i++)
      for (const int *c : cols) out.push_back(c[i]);
  };
  std::vector<int> t;
  interleave(t, {prm->BondHAt1, prm->BondHAt2, prm->BondHNum}, prm->Nbonh);
  write_ints(fp, "BONDS_INC_HYDROGEN", t.data(), static_cast<long>(t.size()));
  interleave(t, {prm->BondAt1, prm->BondAt2, prm->BondNum}, prm->Nbona);
  write_ints(fp, "BONDS_WITHOUT_HYDROGEN", t.data(), static_cast<long>(t.size()));
  interleave(t, {prm->AngleHAt1, prm->AngleHAt2, prm->AngleHAt3, prm->AngleHNum}, prm->Ntheth);
  write_ints(fp, "ANGLES_INC_HYDROGEN", t.data(), static_cast<long>(t.size()));
  interleave(t, {prm->AngleAt1, prm->AngleAt2, prm->AngleAt3, prm->AngleNum}, prm->Ntheta);
  write_ints(fp, "ANGLES_WITHOUT_HYDROGEN", t.data(), static_cast<long>(t.size()));
  interleave(t, {prm->DihHAt1, prm->DihHAt2, prm->DihHAt3, prm->DihHAt4, prm->DihHNum}, prm->Nphih);
  write_ints(fp, "DIHEDRALS_INC_HYDROGEN", t.data(), static_cast<long>(t.size()));
  interleave(t, {prm->DihAt1, prm->DihAt2, prm->DihAt3, prm->DihAt4, prm->DihNum}, prm->Nphia);
  write_ints(fp, "DIHEDRALS_WITHOUT_HYDROGEN", t.data(), static_cast<long>(t.size()));
  write_ints(fp, "EXCLUDED_ATOMS_LIST", prm->ExclAt, prm->Nnb);
  write_reals(fp, "HBOND_ACOEF", prm->HB12, prm->Nphb);
  write_reals(fp, "HBOND_BCOEF", prm->HB10, prm->Nphb);
  {
    std::vector<double> z(prm->Nphb, 0.0);
    write_reals(fp, "HBCUT", z.data(), prm->Nphb);
  }
  write_names(fp, "AMBER_ATOM_TYPE", prm->AtomType, prm->Natom);
  write_names(fp, "TREE_CHAIN_CLASSIFICATION", prm->AtomTree, prm->Natom);
  write_ints(fp, "JOIN_ARRAY", prm->TreeJoin, prm->Natom);
  {
    std::vector<int> z(prm->Natom, 0);
    write_ints(fp, "IROTAT", z.data(), prm->Natom);
  }
  write_section(fp, "RADIUS_SET", "1a80");
  std::fprintf(fp, "%-80s\n", "synthetic intrinsic radii");
  write_reals(fp, "RADII", prm->Rborn, prm->Natom);
  write_reals(fp, "SCREEN", prm->Fs, prm->Natom);
  std::fclose(fp);
  return 0;
}

extern "C" INT_T getxv(STRING_T *fname, INT_T natom, REAL_T start_time, REAL_T *x, REAL_T *v) {
  (void)start_time;
  FILE *fp = (!fname[0] || std::strcmp(fname, "-") == 0) ? stdin : std::fopen(fname, "r");
  if (!fp) {
    std::fprintf(stderr, "getxv: can't open file %s\n", fname);
    std::exit(1);
  }
  char line[256], field[13];
  if (!std::fgets(line, sizeof line, fp) || !std::fgets(line, sizeof line, fp)) {
    std::fprintf(stderr, "getxv: %s is truncated\n", fname);
    std::exit(1);
  }
  int nfile = 0;
  std::sscanf(line, "%d", &nfile);
  if (nfile > 0) natom = nfile;
  auto read_block = [&](double *dst) -> bool {
    for (int i = 0; i < 3 * natom; i++) {
      if (i % 6 == 0 && !std::fgets(line, sizeof line, fp)) return false;
      size_t len = std::strlen(line);
      size_t off = static_cast<size_t>(12 * (i % 6));
      if (off >= len) return false;
      std::memset(field, 0, sizeof field);
      std::strncpy(field, line + off, 12);
      dst[i] = std::atof(field);
    }
    return true;
  };
  if (!read_block(x)) {
    std::fprintf(stderr, "getxv: %s has fewer than %d atoms\n", fname, natom);
    std::exit(1);
  }
  if (v && !read_block(v)) {
    for (int i = 0; i < 3 * natom; i++) v[i] = 0.0;
  }
  if (fp != stdin) std::fclose(fp);
  return 0;
}

extern "C" INT_T putxv(STRING_T *fname, STRING_T *title, INT_T natom, REAL_T start_time,
                       REAL_T *x, REAL_T *v) {
  FILE *fp = std::fopen(fname, "w");
  if (!fp) {
    std::fprintf(stderr, "putxv: can't open file %s\n", fname);
    return 1;
  }
  std::fprintf(fp, "%s\n%5d  %10.5f\n", title ? title : "", natom, start_time);
  auto write_block = [&](const double *src) {
    for (int i = 0; i < 3 * natom; i++) {
      std::fprintf(fp, "%12.7f", src[i]);
      if ((i + 1) % 6 == 0 || i + 1 == 3 * natom) std::fputc('\n', fp);
    }
  };
  write_block(x);
  if (v) write_block(v);
  std::fclose(fp);
  return 0;
}
