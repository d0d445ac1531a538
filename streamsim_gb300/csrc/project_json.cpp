// project_json.cpp — the XML view of a project.json, so that the project
// loader reads a project in its JSON form too.
//
// Restates the reference's ProjectJson accessors (models/histream/src/base/
// projectjson.cpp:45-216: load, resolve, runtimeDefinedDirectory,
// meteorologyPath, numbers, names, string, number, integer, boolean,
// sensorBands) and facetInputView with its helpers
// (models/histream/src/facetrt/facetrtcore.cpp:1846-2036: xmlEscaped, joined,
// joinedNames).  The reference parses the file with nlohmann::json; this
// file has its own small JSON reader with the same value model (objects,
// arrays, strings, integer and floating numbers, booleans, null).  Numbers
// are written into the XML with the standard stream's default format, as
// the reference writes them.
#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <iterator>
#include <map>
#include <memory>
#include <set>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/facetcu.h"

void facetcu_set_host_error(const std::string& message);

namespace facetcu {
namespace project {
namespace {

// ---- JSON values -------------------------------------------------------------
struct Json {
    enum Kind { null, boolean, integer, floating, string, array, object } kind = null;
    bool b = false;
    int64_t i = 0;
    double d = 0.0;
    std::string s;
    std::vector<Json> items;
    std::vector<std::pair<std::string, Json>> members;  // in file order

    bool is_object() const { return kind == object; }
    bool is_array() const { return kind == array; }
    bool is_string() const { return kind == string; }
    bool is_number() const { return kind == integer || kind == floating; }
    float as_float() const { return kind == integer ? float(i) : float(d); }
    const Json* find(const char* key) const
    {
        if (kind != object) return nullptr;
        for (const auto& m : members)
            if (m.first == key) return &m.second;
        return nullptr;
    }
    bool empty() const
    {
        return kind == null || (kind == object && members.empty()) || (kind == array && items.empty());
    }
    std::string dump() const;
};

void dump_string(const std::string& s, std::string& out)
{
    out += '"';
    for (unsigned char ch : s) {
        if (ch == '"' || ch == '\\') {
            out += '\\';
            out += char(ch);
        } else if (ch < 0x20) {
            char buf[8];
            std::snprintf(buf, sizeof(buf), "\\u%04x", ch);
            out += buf;
        } else {
            out += char(ch);
        }
    }
    out += '"';
}

void dump_into(const Json& v, std::string& out)
{
    switch (v.kind) {
    case Json::null: out += "null"; break;
    case Json::boolean: out += v.b ? "true" : "false"; break;
    case Json::integer: out += std::to_string(v.i); break;
    case Json::floating: {
        char buf[32];
        std::snprintf(buf, sizeof(buf), "%.17g", v.d);
        // the shortest representation that reads back to the same double
        for (int p = 1; p <= 17; ++p) {
            char t[32];
            std::snprintf(t, sizeof(t), "%.*g", p, v.d);
            if (std::strtod(t, nullptr) == v.d) {
                std::strcpy(buf, t);
                break;
            }
        }
        out += buf;
        if (!std::strpbrk(buf, ".eEn")) out += ".0";
        break;
    }
    case Json::string: dump_string(v.s, out); break;
    case Json::array:
        out += '[';
        for (size_t k = 0; k < v.items.size(); ++k) {
            if (k) out += ',';
            dump_into(v.items[k], out);
        }
        out += ']';
        break;
    case Json::object:
        out += '{';
        for (size_t k = 0; k < v.members.size(); ++k) {
            if (k) out += ',';
            dump_string(v.members[k].first, out);
            out += ':';
            dump_into(v.members[k].second, out);
        }
        out += '}';
        break;
    }
}

std::string Json::dump() const
{
    std::string out;
    dump_into(*this, out);
    return out;
}

struct Parser {
    const std::string& t;
    size_t at = 0;
    explicit Parser(const std::string& text) : t(text) {}

    [[noreturn]] void fail(const char* what)
    {
        throw std::runtime_error(std::string("Invalid project.json: ") + what + " at offset " +
                                 std::to_string(at));
    }
    void space()
    {
        while (at < t.size() && (t[at] == ' ' || t[at] == '\t' || t[at] == '\n' || t[at] == '\r')) ++at;
    }
    bool take(const char* word)
    {
        const size_t n = std::strlen(word);
        if (t.compare(at, n, word) == 0) {
            at += n;
            return true;
        }
        return false;
    }
    static void utf8(uint32_t cp, std::string& out)
    {
        if (cp < 0x80) {
            out += char(cp);
        } else if (cp < 0x800) {
            out += char(0xC0 | (cp >> 6));
            out += char(0x80 | (cp & 0x3F));
        } else if (cp < 0x10000) {
            out += char(0xE0 | (cp >> 12));
            out += char(0x80 | ((cp >> 6) & 0x3F));
            out += char(0x80 | (cp & 0x3F));
        } else {
            out += char(0xF0 | (cp >> 18));
            out += char(0x80 | ((cp >> 12) & 0x3F));
            out += char(0x80 | ((cp >> 6) & 0x3F));
            out += char(0x80 | (cp & 0x3F));
        }
    }
    uint32_t hex4()
    {
        if (at + 4 > t.size()) fail("short \\u escape");
        uint32_t v = 0;
        for (int k = 0; k < 4; ++k) {
            const char ch = t[at++];
            v <<= 4;
            if (ch >= '0' && ch <= '9') v |= uint32_t(ch - '0');
            else if (ch >= 'a' && ch <= 'f') v |= uint32_t(ch - 'a' + 10);
            else if (ch >= 'A' && ch <= 'F') v |= uint32_t(ch - 'A' + 10);
            else fail("bad \\u escape");
        }
        return v;
    }
    std::string str()
    {
        if (t[at] != '"') fail("expected a string");
        ++at;
        std::string out;
        while (true) {
            if (at >= t.size()) fail("unterminated string");
            const char ch = t[at++];
            if (ch == '"') break;
            if (ch != '\\') {
                out += ch;
                continue;
            }
            if (at >= t.size()) fail("unterminated escape");
            const char e = t[at++];
            switch (e) {
            case '"': out += '"'; break;
            case '\\': out += '\\'; break;
            case '/': out += '/'; break;
            case 'b': out += '\b'; break;
            case 'f': out += '\f'; break;
            case 'n': out += '\n'; break;
            case 'r': out += '\r'; break;
            case 't': out += '\t'; break;
            case 'u': {
                uint32_t cp = hex4();
                if (cp >= 0xD800 && cp < 0xDC00 && take("\\u")) {
                    const uint32_t lo = hex4();
                    cp = 0x10000 + ((cp - 0xD800) << 10) + (lo - 0xDC00);
                }
                utf8(cp, out);
                break;
            }
            default: fail("bad escape");
            }
        }
        return out;
    }
    Json value()
    {
        space();
        if (at >= t.size()) fail("unexpected end");
        Json v;
        const char ch = t[at];
        if (ch == '{') {
            ++at;
            v.kind = Json::object;
            space();
            if (at < t.size() && t[at] == '}') {
                ++at;
                return v;
            }
            while (true) {
                space();
                std::string key = str();
                space();
                if (at >= t.size() || t[at] != ':') fail("expected ':'");
                ++at;
                Json item = value();
                bool replaced = false;  // a repeated key keeps the last value
                for (auto& m : v.members)
                    if (m.first == key) {
                        m.second = item;
                        replaced = true;
                    }
                if (!replaced) v.members.emplace_back(std::move(key), std::move(item));
                space();
                if (at < t.size() && t[at] == ',') {
                    ++at;
                    continue;
                }
                if (at < t.size() && t[at] == '}') {
                    ++at;
                    break;
                }
                fail("expected ',' or '}'");
            }
        } else if (ch == '[') {
            ++at;
            v.kind = Json::array;
            space();
            if (at < t.size() && t[at] == ']') {
                ++at;
                return v;
            }
            while (true) {
                v.items.push_back(value());
                space();
                if (at < t.size() && t[at] == ',') {
                    ++at;
                    continue;
                }
                if (at < t.size() && t[at] == ']') {
                    ++at;
                    break;
                }
                fail("expected ',' or ']'");
            }
        } else if (ch == '"') {
            v.kind = Json::string;
            v.s = str();
        } else if (take("true")) {
            v.kind = Json::boolean;
            v.b = true;
        } else if (take("false")) {
            v.kind = Json::boolean;
        } else if (take("null")) {
            v.kind = Json::null;
        } else {
            const size_t start = at;
            if (at < t.size() && t[at] == '-') ++at;
            bool fraction = false;
            while (at < t.size() && (std::isdigit(static_cast<unsigned char>(t[at])) || t[at] == '.' ||
                                     t[at] == 'e' || t[at] == 'E' || t[at] == '+' || t[at] == '-')) {
                if (t[at] == '.' || t[at] == 'e' || t[at] == 'E') fraction = true;
                ++at;
            }
            const std::string num = t.substr(start, at - start);
            if (num.empty() || num == "-") fail("unexpected character");
            if (!fraction) {
                errno = 0;
                char* end = nullptr;
                const long long x = std::strtoll(num.c_str(), &end, 10);
                if (errno == 0 && end && *end == 0) {
                    v.kind = Json::integer;
                    v.i = x;
                    return v;
                }
            }
            char* end = nullptr;
            v.kind = Json::floating;
            v.d = std::strtod(num.c_str(), &end);
            if (!end || *end) fail("bad number");
        }
        return v;
    }
};

const Json& empty_object()
{
    static const Json v = [] {
        Json j;
        j.kind = Json::object;
        return j;
    }();
    return v;
}

const Json& empty_array()
{
    static const Json v = [] {
        Json j;
        j.kind = Json::array;
        return j;
    }();
    return v;
}

const Json& object_member(const Json& v, const char* key)
{
    const Json* f = v.find(key);
    return f && f->is_object() ? *f : empty_object();
}

const Json& array_member(const Json& v, const char* key)
{
    const Json* f = v.find(key);
    return f && f->is_array() ? *f : empty_array();
}

float clean(float v, float fallback) { return std::isfinite(v) ? v : fallback; }

std::string jstring(const Json& o, const char* key, const std::string& fallback = {})
{
    const Json* f = o.find(key);
    if (!f) return fallback;
    if (f->is_string()) return f->s;
    return f->kind == Json::null ? fallback : f->dump();
}

float jnumber(const Json& o, const char* key, float fallback)
{
    const Json* f = o.find(key);
    if (!f) return fallback;
    try {
        if (f->is_number()) return clean(f->as_float(), fallback);
        if (f->is_string()) return clean(std::stof(f->s), fallback);
    } catch (...) {
    }
    return fallback;
}

int jinteger(const Json& o, const char* key, int fallback)
{
    return int(std::lround(jnumber(o, key, float(fallback))));
}

bool jboolean(const Json& o, const char* key, bool fallback)
{
    const Json* f = o.find(key);
    if (!f) return fallback;
    if (f->kind == Json::boolean) return f->b;
    if (f->kind == Json::integer) return int(f->i) != 0;
    if (f->is_string()) return f->s == "true" || f->s == "1";
    return fallback;
}

std::vector<float> jnumbers(const Json& v)
{
    std::vector<float> out;
    if (v.is_array()) {
        for (const Json& x : v.items)
            if (x.is_number()) out.push_back(x.as_float());
        return out;
    }
    std::string text;
    if (v.is_string()) text = v.s;
    else if (v.is_number()) text = v.dump();
    std::replace(text.begin(), text.end(), ';', ',');
    std::replace(text.begin(), text.end(), ' ', ',');
    std::istringstream in(text);
    std::string token;
    while (std::getline(in, token, ',')) {
        if (token.empty()) continue;
        try {
            const float x = std::stof(token);
            if (std::isfinite(x)) out.push_back(x);
        } catch (...) {
        }
    }
    return out;
}

struct ProjectFile {
    Json root, configuration;
    std::filesystem::path input;

    std::filesystem::path directory() const { return input.parent_path(); }
    static std::filesystem::path executable_directory() { return std::filesystem::current_path(); }
    std::filesystem::path resolve(const std::string& value) const
    {
        if (value.empty()) return {};
        const std::filesystem::path p(value);
        if (p.is_absolute()) return p.lexically_normal();
        const std::filesystem::path local = (directory() / p).lexically_normal();
        if (std::filesystem::exists(local) || p.begin() == p.end() || *p.begin() != "assets")
            return local;
        for (std::filesystem::path parent = executable_directory(); !parent.empty();
             parent = parent.parent_path()) {
            const std::filesystem::path candidate = (parent / p).lexically_normal();
            if (std::filesystem::exists(candidate)) return candidate;
            if (parent == parent.root_path()) break;
        }
        return local;
    }
    const Json& scene() const { return object_member(configuration, "scene"); }
    const Json& light() const { return object_member(configuration, "light"); }
    const Json& sensor() const { return object_member(configuration, "sensor"); }
    const Json& control() const { return object_member(configuration, "control"); }
    const Json& objects() const { return array_member(object_member(configuration, "objects"), "items"); }
    const Json& spectra() const { return array_member(configuration, "spectra"); }
    const Json& thermals() const { return array_member(configuration, "thermals"); }
    const Json& materials() const { return array_member(configuration, "materials"); }
    const Json& meteorology() const { return object_member(configuration, "meteo"); }
    std::filesystem::path output_directory() const { return resolve(jstring(configuration, "outDir", "output")); }
    std::filesystem::path defined() const { return executable_directory() / "defined"; }
    std::filesystem::path meteorology_path() const
    {
        const std::string v = jstring(meteorology(), "path", "defined/meteo.txt");
        if (v.empty() || v == "defined/meteo.txt" || v == "HiStream \xe5\x86\x85\xe7\xbd\xae\xe6\xb0\x94\xe8\xb1\xa1\xe6\x95\xb0\xe6\x8d\xae")
            return defined() / "meteo.txt";
        return resolve(v);
    }
    std::vector<float> sensor_bands() const
    {
        std::vector<float> values;
        std::set<long long> keys;
        auto add = [&](float v) {
            if (!(v > 0.0f) || !std::isfinite(v)) return;
            const long long key = std::llround(v * 1000000.0);
            if (keys.insert(key).second) values.push_back(v);
        };
        const Json* bands = sensor().find("bands");
        const std::vector<float> custom = bands ? jnumbers(*bands) : std::vector<float>{};
        if (jboolean(sensor(), "continuousBands", false)) {
            const float start = jnumber(sensor(), "bandStart", 400.0f);
            const float end = jnumber(sensor(), "bandEnd", 2500.0f);
            const float step = jnumber(sensor(), "bandStep", 10.0f);
            if (start > 0.0f && end >= start && step > 0.0f)
                for (int k = 0; k < 800 && start + k * step <= end + 1e-5f; ++k) add(start + k * step);
        }
        for (float v : custom) add(v);
        if (values.empty()) values.push_back(10500.0f);
        std::sort(values.begin(), values.end());
        if (values.size() > 800) values.resize(800);
        return values;
    }
};

ProjectFile load_file(const std::string& path)
{
    if (path.empty()) throw std::invalid_argument("project.json path is required");
    ProjectFile pf;
    pf.input = std::filesystem::absolute(path).lexically_normal();
    std::string name = pf.input.filename().string();
    std::transform(name.begin(), name.end(), name.begin(),
                   [](unsigned char ch) { return char(std::tolower(ch)); });
    if (name != "project.json") throw std::invalid_argument("HiStream accepts project.json only");
    std::ifstream in(pf.input, std::ios::binary);
    if (!in) throw std::runtime_error("Cannot open project.json: " + pf.input.string());
    const std::string text{std::istreambuf_iterator<char>(in), std::istreambuf_iterator<char>()};
    Parser parser(text);
    pf.root = parser.value();
    parser.space();
    if (parser.at != text.size()) parser.fail("trailing characters");
    if (!pf.root.is_object()) throw std::runtime_error("project.json root must be an object");
    const std::string format = jstring(pf.root, "format", "streamsim-project");
    if (format != "streamsim-project") throw std::runtime_error("Unsupported project format: " + format);
    const int version = jinteger(pf.root, "schemaVersion", 1);
    if (version < 1 || version > 6)
        throw std::runtime_error("Unsupported project schemaVersion; expected 1-6");
    pf.configuration = object_member(pf.root, "configuration");
    if (pf.configuration.empty()) throw std::runtime_error("project.json has no configuration object");
    return pf;
}

std::string escaped(std::string v)
{
    const std::pair<const char*, const char*> entities[] = {
        {"&", "&amp;"}, {"<", "&lt;"}, {">", "&gt;"}, {"\"", "&quot;"}, {"'", "&apos;"}};
    for (const auto& e : entities) {
        size_t at = 0;
        while ((at = v.find(e.first, at)) != std::string::npos) {
            v.replace(at, std::strlen(e.first), e.second);
            at += std::strlen(e.second);
        }
    }
    return v;
}

std::string joined(const std::vector<float>& v)
{
    std::ostringstream out;
    for (size_t k = 0; k < v.size(); ++k) {
        if (k) out << ',';
        out << v[k];
    }
    return out.str();
}

std::string joined_names(const Json& object, const char* key, const std::string& fallback)
{
    std::ostringstream out;
    const Json* meshes = object.find("meshes");
    if (meshes && meshes->is_array()) {
        size_t k = 0;
        for (const Json& m : meshes->items) {
            if (k++) out << ',';
            out << jstring(m, key, fallback);
        }
    }
    return out.str().empty() ? fallback : out.str();
}

}  // namespace

// facetInputView (facetrtcore.cpp:1888-2036)
std::string xml_view(const std::string& path)
{
    const ProjectFile project = load_file(path);
    const Json& scene = project.scene();
    const Json& light = project.light();
    const Json& sensor = project.sensor();
    const Json& control = project.control();
    const Json& meteo = project.meteorology();
    const Json* bg = scene.find("background");
    const Json& background = bg ? *bg : empty_object();
    for (const Json& m : project.materials().items)
        if (jstring(m, "energyModel") == "photovoltaic" &&
            jstring(m, "name") == jstring(background, "materialName"))
            throw std::runtime_error("Photovoltaic panels must be scene objects, not background ground");
    const std::filesystem::path defined = project.defined();
    std::ostringstream x;
    x << "<HiStreamProject><Control>"
      << "<outDir>" << escaped(project.output_directory().string()) << "</outDir>"
      << "<facetBackend>" << escaped(jstring(control, "facetBackend", "gpu")) << "</facetBackend>"
      << "<GPU>" << jinteger(control, "gpu", 0) << "</GPU>"
      << "<rayTracingDepth>" << jinteger(control, "depth", 4) << "</rayTracingDepth>"
      << "<periodicNeighborCount>"
      << std::clamp(jinteger(control, "periodicTraversalCount",
                             jboolean(control, "periodicBoundary", false)
                                 ? jinteger(control, "periodicNeighborCount", 8)
                                 : 0),
                    0, 20)
      << "</periodicNeighborCount>"
      << "<couplingIterations>" << jinteger(control, "couplingIterations", 20) << "</couplingIterations>"
      << "<temperatureTolerance>" << jnumber(control, "temperatureTolerance", 0.05f) << "</temperatureTolerance>"
      << "<temperatureRelaxation>" << jnumber(control, "temperatureRelaxation", 0.5f) << "</temperatureRelaxation>"
      << "<spectralAccelerationWidth>" << jnumber(control, "spectralAccelerationWidth", 100.0f) << "</spectralAccelerationWidth>"
      << "<radiationSolver>" << escaped(jstring(control, "radiationSolver", "traditional")) << "</radiationSolver>"
      << "<vegetationTemperatureMethod>" << jinteger(control, "vegetationTemperatureMethod", 0) << "</vegetationTemperatureMethod>"
      << "<isDEM>" << (jboolean(scene, "terrain", false) ? 1 : 0) << "</isDEM>"
      << "<isProcess>" << (jboolean(sensor, "process", false) ? 1 : 0) << "</isProcess>"
      << "<isRadiationProcess>" << (jboolean(sensor, "radiationProcess", false) ? 1 : 0) << "</isRadiationProcess>"
      << "<isEnergyProcess>" << (jboolean(sensor, "energyProcess", false) ? 1 : 0) << "</isEnergyProcess>"
      << "</Control><Geometry><Light><light name=\"Solar\">"
      << "<lightAngle><viewAngles>" << jnumber(light, "zenith", 30.0f) << ','
      << jnumber(light, "azimuth", 135.0f) << "</viewAngles></lightAngle>"
      << "<skyTemperature>" << jnumber(light, "skyTemperature", 250.0f) << "</skyTemperature>"
      << "<directScatteringRatio>" << jnumber(light, "direct", 0.8f) << "</directScatteringRatio>"
      << "<esunFileName>" << escaped((defined / "Esun_.dat").string()) << "</esunFileName>"
      << "<eskyFileName>" << escaped((defined / "Esky_.dat").string()) << "</eskyFileName>"
      << "</light></Light><Sensor><sensor name=\"MainSensor\">"
      << "<controlBand>" << joined(project.sensor_bands()) << "</controlBand>"
      << "</sensor></Sensor></Geometry><Scene>"
      << "<sceneSizeX>" << jnumber(scene, "x", 60.0f) << "</sceneSizeX>"
      << "<sceneSizeY>" << jnumber(scene, "y", 60.0f) << "</sceneSizeY>"
      << "<Height>" << jnumber(scene, "height", 15.0f) << "</Height>"
      << "<voxelSize>" << jnumber(scene, "voxel", 1.0f) << "</voxelSize>"
      << "<bgSpectral>" << escaped(jstring(background, "spectralName", "soil")) << "</bgSpectral>"
      << "<bgThermal>" << escaped(jstring(background, "thermalName", "soil_temperature")) << "</bgThermal>"
      << "<bgBioName>" << escaped(jstring(background, "materialName", "soilset")) << "</bgBioName>"
      << "<backgroundHeterogeneity>" << (jboolean(background, "heterogeneityEnabled", false) ? "Hapke" : "Lambert") << "</backgroundHeterogeneity>"
      << "<backgroundAngularStrength>" << jnumber(background, "angularEffectStrength", 0.5f) << "</backgroundAngularStrength>";
    if (jboolean(scene, "terrain", false) && !jstring(scene, "demFile").empty())
        x << "<DEM>" << escaped(project.resolve(jstring(scene, "demFile")).string()) << "</DEM>";
    x << "<Object>";
    for (const Json& object : project.objects().items) {
        const std::string type = jstring(object, "type", "Vegetation");
        if (type == "Fire" || type == "Fog" || object.find("medium")) continue;
        const std::string name = jstring(object, "name", "object");
        const std::string spectral = jstring(object, "spectralName", "soil");
        const std::string thermal = jstring(object, "thermalName", "soil_temperature");
        const std::string canopy = jstring(object, "canopyName", type == "Vegetation" ? "canopy_default" : "rigid_body");
        const std::string material = jstring(object, "materialName",
                                             type == "Vegetation" ? "leaf_c3" : type == "Water" ? "water_set" : "soilset");
        const Json* dims = object.find("dimensions");
        std::vector<float> d = jnumbers(dims ? *dims : empty_array());
        while (d.size() < 3) d.push_back(1.0f);
        x << "<object objName=\"" << escaped(name) << "\">"
          << "<componentType>" << escaped(type) << "</componentType>"
          << "<meshNames>" << escaped(joined_names(object, "name", name)) << "</meshNames>"
          << "<spectralNames>" << escaped(joined_names(object, "spectralName", spectral)) << "</spectralNames>"
          << "<thermalNames>" << escaped(joined_names(object, "thermalName", thermal)) << "</thermalNames>"
          << "<canopyNames>" << escaped(joined_names(object, "canopyName", canopy)) << "</canopyNames>"
          << "<bioNames>" << escaped(joined_names(object, "materialName", material)) << "</bioNames>"
          << "<propNames>" << escaped(joined_names(object, "materialName", material)) << "</propNames>"
          << "<shapes>" << d[0] << ',' << d[1] << ',' << d[2] << "</shapes>";
        const std::string model = jstring(object, "fileName");
        const std::string positions = jstring(object, "positionFile");
        if (!model.empty()) x << "<fileName>" << escaped(project.resolve(model).string()) << "</fileName>";
        if (!positions.empty()) x << "<objectPosition>" << escaped(project.resolve(positions).string()) << "</objectPosition>";
        x << "</object>";
    }
    x << "</Object></Scene><Attribute><Optical>";
    for (const Json& item : project.spectra().items) {
        const Json* pr = item.find("params");
        const Json& params = pr ? *pr : empty_object();
        const Json* tx = item.find("physicalTexture");
        const Json& texture = tx ? *tx : empty_object();
        x << "<spectral name=\"" << escaped(jstring(item, "name", "spectral")) << "\" type=\""
          << escaped(jstring(item, "model", "custom")) << "\">"
          << "<reflectance>" << escaped(jstring(item, "reflectance", "0.2")) << "</reflectance>"
          << "<transmittance>" << escaped(jstring(item, "transmittance", "0")) << "</transmittance>"
          << "<ref_TIR>" << jnumber(item, "refTir", 0.05f) << "</ref_TIR>"
          << "<tau_TIR>" << jnumber(item, "tauTir", 0.0f) << "</tau_TIR>"
          << "<Cab>" << jnumber(params, "Cab", 40) << "</Cab><Cw>" << jnumber(params, "Cw", .01f)
          << "</Cw><Cdm>" << jnumber(params, "Cdm", .01f) << "</Cdm><Cs>" << jnumber(params, "Cs", 0)
          << "</Cs><N>" << jnumber(params, "N", 1.5f) << "</N><SMC>" << jnumber(params, "SMC", 25)
          << "</SMC><BSMBrightness>" << jnumber(params, "BSMBrightness", .5f) << "</BSMBrightness><BSMlat>"
          << jnumber(params, "BSMlat", 25) << "</BSMlat><BSMlon>" << jnumber(params, "BSMlon", 45) << "</BSMlon>"
          << "<physicalTextureEnabled>" << (jboolean(texture, "enabled", false) ? 1 : 0) << "</physicalTextureEnabled>"
          << "<physicalTextureStrength>" << jnumber(texture, "strength", 0.2f) << "</physicalTextureStrength>"
          << "<physicalTextureRepeatSize>" << jnumber(texture, "repeatSize", 2.0f) << "</physicalTextureRepeatSize>";
        if (!jstring(texture, "fileName").empty())
            x << "<physicalTextureFile>" << escaped(project.resolve(jstring(texture, "fileName")).string()) << "</physicalTextureFile>";
        if (!jstring(item, "fileName").empty())
            x << "<spectral_file>" << escaped(project.resolve(jstring(item, "fileName")).string()) << "</spectral_file>";
        x << "</spectral>";
    }
    x << "</Optical><Thermal>";
    for (const Json& item : project.thermals().items)
        x << "<thermal name=\"" << escaped(jstring(item, "name", "temperature")) << "\"><sunlitTemperature>"
          << jnumber(item, "sunlitTemperature", 305) << "</sunlitTemperature><shadedTemperature>"
          << jnumber(item, "shadedTemperature", 295) << "</shadedTemperature></thermal>";
    x << "</Thermal><Biochemistry>";
    for (const Json& item : project.materials().items) {
        if (jstring(item, "type", "Soil") != "Soil") continue;
        const Json* pr = item.find("params");
        const Json& params = pr ? *pr : empty_object();
        x << "<property><soilSet name=\"" << escaped(jstring(item, "name", "soilset")) << "\">"
          << "<method>" << jinteger(control, "soilTemperatureMethod", jinteger(params, "method", 1)) << "</method>"
          << "<rss>" << jnumber(params, "rss", 2000) << "</rss><cs>" << jnumber(params, "cs", 1180)
          << "</cs><rhos>" << jnumber(params, "rhos", 1800) << "</rhos><lambdas>"
          << jnumber(params, "lambdas", 1.55f) << "</lambdas><SMC>" << jnumber(params, "SMC", 25)
          << "</SMC></soilSet></property>";
    }
    for (const Json& item : project.materials().items) {
        const Json* pr = item.find("params");
        const Json& p = pr ? *pr : empty_object();
        const bool pv = jstring(item, "energyModel") == "photovoltaic";
        x << "<surfaceEnergy name=\"" << escaped(jstring(item, "name")) << "\">"
          << "<photovoltaic>" << (pv ? 1 : 0) << "</photovoltaic>"
          << "<vegetation>" << (jstring(item, "type") == "Vegetation" && jstring(item, "energyModel") != "wood" ? 1 : 0) << "</vegetation>"
          << "<eta25>" << jnumber(p, "eta25", .22f) << "</eta25>"
          << "<gamma>" << jnumber(p, "gamma", -.0035f) << "</gamma>"
          << "<bifaciality>" << jnumber(p, "bifaciality", 0) << "</bifaciality>"
          << "<heatCapacityPerArea>" << jnumber(p, "heatCapacityPerArea", pv ? 12000 : 60000) << "</heatCapacityPerArea>"
          << "<convectiveScale>" << jnumber(p, "convectiveScale", 1) << "</convectiveScale></surfaceEnergy>";
    }
    x << "</Biochemistry></Attribute><Meteorology>"
      << "<filePath>" << escaped(project.meteorology_path().string()) << "</filePath>"
      << "<startTimeNode>" << jinteger(meteo, "start", 0) << "</startTimeNode>"
      << "<endTimeNode>" << jinteger(meteo, "end", 1) << "</endTimeNode>"
      << "<dTime>" << jnumber(meteo, "dTime", 1800) << "</dTime>"
      << "<Latitude>" << jnumber(meteo, "latitude", 40) << "</Latitude>"
      << "<Longitude>" << jnumber(meteo, "longitude", 116) << "</Longitude>"
      << "</Meteorology></HiStreamProject>";
    return x.str();
}

}  // namespace project
}  // namespace facetcu

extern "C" {

int facetcu_project_xml_view(const char* path, char* buffer, uint64_t capacity, uint64_t* length)
{
    facetcu_set_host_error("");
    if (!path || !length) {
        facetcu_set_host_error("path and length are required");
        return FACETCU_INVALID_ARGUMENT;
    }
    try {
        const std::string xml = facetcu::project::xml_view(path);
        *length = xml.size();
        if (buffer && capacity) {
            const size_t n = std::min<size_t>(xml.size(), size_t(capacity - 1));
            std::memcpy(buffer, xml.data(), n);
            buffer[n] = 0;
        }
        if (capacity && xml.size() >= capacity) {
            facetcu_set_host_error("buffer too small for the XML view");
            return FACETCU_OVERFLOW_ERROR;
        }
        return FACETCU_OK;
    } catch (const std::invalid_argument& e) {
        facetcu_set_host_error(e.what());
        return FACETCU_INVALID_ARGUMENT;
    } catch (const std::exception& e) {
        facetcu_set_host_error(e.what());
        return FACETCU_RUNTIME_ERROR;
    }
}

}  // extern "C"
