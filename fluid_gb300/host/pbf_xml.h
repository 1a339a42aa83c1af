// Particle files in the reference's XML format (Application::load_particles,
// src/application.cpp:302-344):
//
//   <particles>
//     <density>rho0</density>
//     <ps> <particle><pos>x y z</pos><v>vx vy vz</v></particle> ... </ps>
//     <fs/>
//   </particles>
//
// plus an optional <params> element (h, h2, iters, scorr_n, epsilon, scorr_k,
// scorr_dq, vort_eps, xsph_c, dt, gravity, box_lo, box_hi, box_open_mask)
// that the reference's loader ignores. A small self-contained XML reader:
// elements, text, attributes (skipped), comments, the <?xml?> prolog and the
// five predefined entities.
#pragma once

#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "pbf.h"

namespace pbf_host {

struct XmlNode {
  std::string name;
  std::string text;  // concatenated character data directly inside this element
  std::vector<std::unique_ptr<XmlNode>> children;
  const XmlNode* child(const std::string& n) const;
  std::vector<const XmlNode*> children_named(const std::string& n) const;
};

class XmlError : public std::runtime_error {
 public:
  using std::runtime_error::runtime_error;
};

// Parse a whole document; throws XmlError with a line number on malformed input.
std::unique_ptr<XmlNode> parse_xml(const std::string& text);

struct ParticleFile {
  double rest_density = 1000.0;     // Particles(double rest_density = 1000.0)
  std::vector<double> pos, vel;     // (n, 3) row-major
  pbf_params params{};              // reference defaults, rest_density and <params> applied
  bool has_params = false;
  size_t size() const { return pos.size() / 3; }
};

enum class LoadStatus { ok, missing, xml_error, not_particles };

// Load like Application::load_particles: a missing file gives an empty set with
// the default rest density; <density> goes through float (stof). `message`
// receives the reason for any status other than ok.
LoadStatus load_particle_file(const std::string& path, ParticleFile* out, std::string* message);

// Write a particle file (with <params> when params is given).
bool write_particle_file(const std::string& path, double rest_density, const std::vector<double>& pos,
                         const std::vector<double>& vel, const pbf_params* params);

}  // namespace pbf_host
