#include "pbf_xml.h"

#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iomanip>
#include <sstream>

namespace pbf_host {

const XmlNode* XmlNode::child(const std::string& n) const {
  for (const auto& c : children)
    if (c->name == n) return c.get();
  return nullptr;
}

std::vector<const XmlNode*> XmlNode::children_named(const std::string& n) const {
  std::vector<const XmlNode*> out;
  for (const auto& c : children)
    if (c->name == n) out.push_back(c.get());
  return out;
}

namespace {

class Reader {
 public:
  explicit Reader(const std::string& s) : s_(s) {}

  std::unique_ptr<XmlNode> document() {
    skip_misc();
    if (!at('<')) fail("expected the root element");
    auto root = element();
    skip_misc();
    if (p_ != s_.size()) fail("content after the root element");
    return root;
  }

 private:
  const std::string& s_;
  size_t p_ = 0;

  [[noreturn]] void fail(const std::string& what) const {
    size_t line = 1;
    for (size_t i = 0; i < p_ && i < s_.size(); ++i) line += s_[i] == '\n';
    throw XmlError("XML error at line " + std::to_string(line) + ": " + what);
  }
  bool at(char c) const { return p_ < s_.size() && s_[p_] == c; }
  bool starts(const char* t) const { return s_.compare(p_, std::char_traits<char>::length(t), t) == 0; }
  static bool space(char c) { return c == ' ' || c == '\t' || c == '\n' || c == '\r'; }
  static bool name_char(char c) {
    return (c >= 'a' && c <= 'z') || (c >= 'A' && c <= 'Z') || (c >= '0' && c <= '9') || c == '_' || c == '-' ||
           c == '.' || c == ':';
  }
  void skip_space() {
    while (p_ < s_.size() && space(s_[p_])) ++p_;
  }
  void skip_until(const char* end) {
    const size_t q = s_.find(end, p_);
    if (q == std::string::npos) fail(std::string("unterminated construct, expected ") + end);
    p_ = q + std::char_traits<char>::length(end);
  }
  // prolog, comments, processing instructions, doctype and whitespace
  void skip_misc() {
    for (;;) {
      skip_space();
      if (starts("<?")) skip_until("?>");
      else if (starts("<!--")) skip_until("-->");
      else if (starts("<!")) skip_until(">");
      else return;
    }
  }
  std::string name() {
    const size_t b = p_;
    while (p_ < s_.size() && name_char(s_[p_])) ++p_;
    if (p_ == b) fail("expected a name");
    return s_.substr(b, p_ - b);
  }
  void append_text(std::string* out, size_t b, size_t e) {
    for (size_t i = b; i < e; ++i) {
      if (s_[i] != '&') {
        out->push_back(s_[i]);
        continue;
      }
      const size_t semi = s_.find(';', i);
      if (semi == std::string::npos || semi > e) fail("bad entity");
      const std::string ent = s_.substr(i + 1, semi - i - 1);
      if (ent == "lt") out->push_back('<');
      else if (ent == "gt") out->push_back('>');
      else if (ent == "amp") out->push_back('&');
      else if (ent == "quot") out->push_back('"');
      else if (ent == "apos") out->push_back('\'');
      else if (!ent.empty() && ent[0] == '#') {
        const long v = std::strtol(ent.c_str() + 1 + (ent.size() > 1 && ent[1] == 'x'), nullptr,
                                   (ent.size() > 1 && ent[1] == 'x') ? 16 : 10);
        out->push_back(static_cast<char>(v & 0x7f));
      } else {
        fail("unknown entity &" + ent + ";");
      }
      i = semi;
    }
  }
  std::unique_ptr<XmlNode> element() {
    ++p_;  // '<'
    auto node = std::make_unique<XmlNode>();
    node->name = name();
    for (;;) {  // attributes are read and dropped
      skip_space();
      if (starts("/>")) {
        p_ += 2;
        return node;
      }
      if (at('>')) {
        ++p_;
        break;
      }
      name();
      skip_space();
      if (!at('=')) fail("expected '=' in an attribute");
      ++p_;
      skip_space();
      if (!at('"') && !at('\'')) fail("expected a quoted attribute value");
      const char q = s_[p_++];
      const size_t e = s_.find(q, p_);
      if (e == std::string::npos) fail("unterminated attribute value");
      p_ = e + 1;
    }
    for (;;) {  // content
      if (p_ >= s_.size()) fail("unterminated element <" + node->name + ">");
      if (starts("</")) {
        p_ += 2;
        const std::string n = name();
        if (n != node->name) fail("mismatched </" + n + "> for <" + node->name + ">");
        skip_space();
        if (!at('>')) fail("expected '>'");
        ++p_;
        return node;
      }
      if (starts("<!--")) {
        skip_until("-->");
      } else if (starts("<![CDATA[")) {
        p_ += 9;
        const size_t e = s_.find("]]>", p_);
        if (e == std::string::npos) fail("unterminated CDATA");
        node->text.append(s_, p_, e - p_);
        p_ = e + 3;
      } else if (starts("<?")) {
        skip_until("?>");
      } else if (at('<')) {
        node->children.push_back(element());
      } else {
        const size_t b = p_;
        while (p_ < s_.size() && s_[p_] != '<') ++p_;
        append_text(&node->text, b, p_);
      }
    }
  }
};

bool read_vec3(const std::string& text, double out[3]) {
  std::istringstream ss(text);  // Application::stov, application.cpp:292-299
  ss >> out[0] >> out[1] >> out[2];
  return !ss.fail();
}

bool read_number(const XmlNode* n, double* out) {
  if (!n) return false;
  char* end = nullptr;
  errno = 0;
  const double v = std::strtod(n->text.c_str(), &end);
  if (end == n->text.c_str() || errno) return false;
  *out = v;
  return true;
}

void read_params(const XmlNode* p, pbf_params* prm) {
  double v;
  if (read_number(p->child("h"), &v)) prm->h = v;
  if (read_number(p->child("h2"), &v)) prm->h2 = v;
  if (read_number(p->child("iters"), &v)) prm->iters = static_cast<int32_t>(v);
  if (read_number(p->child("scorr_n"), &v)) prm->scorr_n = static_cast<int32_t>(v);
  if (read_number(p->child("epsilon"), &v)) prm->epsilon = v;
  if (read_number(p->child("scorr_k"), &v)) prm->scorr_k = v;
  if (read_number(p->child("scorr_dq"), &v)) prm->scorr_dq = v;
  if (read_number(p->child("vort_eps"), &v)) prm->vort_eps = v;
  if (read_number(p->child("xsph_c"), &v)) prm->xsph_c = v;
  if (read_number(p->child("dt"), &v)) prm->dt = v;
  if (read_number(p->child("box_open_mask"), &v)) prm->box_open_mask = static_cast<int32_t>(v);
  double g[3];
  if (const XmlNode* n = p->child("gravity"))
    if (read_vec3(n->text, g))
      for (int k = 0; k < 3; ++k) prm->gravity[k] = g[k];
  if (const XmlNode* n = p->child("box_lo"))
    if (read_vec3(n->text, g))
      for (int k = 0; k < 3; ++k) prm->box_lo[k] = g[k];
  if (const XmlNode* n = p->child("box_hi"))
    if (read_vec3(n->text, g))
      for (int k = 0; k < 3; ++k) prm->box_hi[k] = g[k];
}

}  // namespace

std::unique_ptr<XmlNode> parse_xml(const std::string& text) { return Reader(text).document(); }

LoadStatus load_particle_file(const std::string& path, ParticleFile* out, std::string* message) {
  *out = ParticleFile();
  pbf_params_default(&out->params);
  std::ifstream f(path, std::ios::binary);
  if (!f) {
    if (message) *message = "particle file not passed in or not found: " + path;
    return LoadStatus::missing;  // application.cpp:303-308: an empty Particles()
  }
  std::stringstream buf;
  buf << f.rdbuf();
  std::unique_ptr<XmlNode> root;
  try {
    root = parse_xml(buf.str());
  } catch (const XmlError& e) {
    if (message) *message = e.what();
    return LoadStatus::xml_error;
  }
  if (root->name != "particles") {
    if (message) *message = "not a particles file: root element is <" + root->name + ">";
    return LoadStatus::not_particles;
  }
  if (const XmlNode* d = root->child("density")) {
    // stof, application.cpp:331: the file's rest density is rounded to float
    out->rest_density = static_cast<double>(std::strtof(d->text.c_str(), nullptr));
  }
  out->params.rest_density = out->rest_density;
  if (const XmlNode* p = root->child("params")) {
    read_params(p, &out->params);
    out->has_params = true;
  }
  if (const XmlNode* ps = root->child("ps")) {
    for (const XmlNode* p : ps->children_named("particle")) {
      double x[3] = {0, 0, 0}, v[3] = {0, 0, 0};
      const XmlNode* pn = p->child("pos");
      const XmlNode* vn = p->child("v");
      if (!pn || !read_vec3(pn->text, x) || (vn && !read_vec3(vn->text, v))) {
        if (message) *message = "a <particle> lacks a readable <pos> or <v>";
        return LoadStatus::xml_error;
      }
      out->pos.insert(out->pos.end(), x, x + 3);
      out->vel.insert(out->vel.end(), v, v + 3);
    }
  }
  return LoadStatus::ok;
}

bool write_particle_file(const std::string& path, double rest_density, const std::vector<double>& pos,
                         const std::vector<double>& vel, const pbf_params* params) {
  std::ofstream f(path);
  if (!f) return false;
  f << std::setprecision(17);
  f << "<particles>\n  <density>" << rest_density << "</density>\n";
  if (params) {
    f << "  <params><h>" << params->h << "</h><h2>" << params->h2 << "</h2><iters>" << params->iters
      << "</iters><scorr_n>" << params->scorr_n << "</scorr_n><epsilon>" << params->epsilon << "</epsilon><scorr_k>"
      << params->scorr_k << "</scorr_k><scorr_dq>" << params->scorr_dq << "</scorr_dq><vort_eps>" << params->vort_eps
      << "</vort_eps><xsph_c>" << params->xsph_c << "</xsph_c><dt>" << params->dt << "</dt><gravity>"
      << params->gravity[0] << ' ' << params->gravity[1] << ' ' << params->gravity[2] << "</gravity><box_lo>"
      << params->box_lo[0] << ' ' << params->box_lo[1] << ' ' << params->box_lo[2] << "</box_lo><box_hi>"
      << params->box_hi[0] << ' ' << params->box_hi[1] << ' ' << params->box_hi[2] << "</box_hi><box_open_mask>"
      << params->box_open_mask << "</box_open_mask></params>\n";
  }
  f << "  <ps>\n";
  for (size_t i = 0; i + 2 < pos.size(); i += 3) {
    f << "    <particle><pos>" << pos[i] << ' ' << pos[i + 1] << ' ' << pos[i + 2] << "</pos><v>" << vel[i] << ' '
      << vel[i + 1] << ' ' << vel[i + 2] << "</v></particle>\n";
  }
  f << "  </ps>\n  <fs/>\n</particles>\n";
  return static_cast<bool>(f);
}

}  // namespace pbf_host
