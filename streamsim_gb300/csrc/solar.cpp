// solar.cpp — the sun of a FacetEB node.
//
// runFacetEBCore places each node's sun with NREL's Solar Position Algorithm
// (the vendored thirdparty/spa.cpp, function SPA_ZA), fed by
// updateSolarPosition (facetrtcore.cpp:3290-3327): the node's day of 2019
// (Utils::calculateMonthAndDay, utils.cpp:615-632), whole minutes of local
// time in UTC+8, Utils::calculateDeltaT (utils.cpp:572-609), 100 m of
// elevation, the node's pressure (at least 100 mbar) and air temperature,
// 0.5667 deg of refraction at the horizon; a failed calculation throws
// "FacetEB solar-position calculation failed".
//
// SPA's periodic-term tables are not restated here.  The sun's coordinates
// come from the formulas of J. Meeus, Astronomical Algorithms (2nd ed.,
// 1998): chapter 7 (Julian day), 12 (sidereal time), 22 (nutation, its four
// main terms), 25 (the sun: mean longitude and anomaly, equation of the
// centre, radius vector, aberration, obliquity) and 40 (topocentric
// parallax), with SPA's published input ranges and error codes and its
// refraction correction (Reda and Andreas, NREL/TP-560-34302, eq. 42-43).
// These agree with SPA to about 0.01 deg in the sun's direction.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <stdexcept>
#include <string>

#include "../../include/facetcu.h"

void facetcu_set_host_error(const std::string& message);

namespace facetcu {
namespace solar {
namespace {

constexpr double kPi = 3.14159265358979323846;
constexpr double kSunRadius = 0.26667;  // degrees

double rad(double d) { return d * kPi / 180.0; }
double deg(double r) { return r * 180.0 / kPi; }
double wrap360(double d)
{
    d = std::fmod(d, 360.0);
    return d < 0.0 ? d + 360.0 : d;
}

// SPA's input checks and error codes for SPA_ZA.
int validate(const facetcu_solar_input& in)
{
    if (in.year < -2000 || in.year > 6000) return 1;
    if (in.month < 1 || in.month > 12) return 2;
    if (in.day < 1 || in.day > 31) return 3;
    if (in.hour < 0 || in.hour > 24) return 4;
    if (in.minute < 0 || in.minute > 59) return 5;
    if (in.second < 0 || in.second > 59) return 6;
    if (in.hour == 24 && in.minute > 0) return 5;
    if (in.hour == 24 && in.second > 0) return 6;
    if (!(std::fabs(in.delta_t) <= 8000.0)) return 7;
    if (!(std::fabs(in.timezone) <= 18.0)) return 8;
    if (!(std::fabs(in.longitude) <= 180.0)) return 9;
    if (!(std::fabs(in.latitude) <= 90.0)) return 10;
    if (!(std::fabs(in.atmos_refract) <= 5.0)) return 16;
    if (!(in.elevation >= -6500000.0)) return 11;
    if (!(in.pressure >= 0.0 && in.pressure <= 5000.0)) return 12;
    if (!(in.temperature > -273.0 && in.temperature <= 6000.0)) return 13;
    return 0;
}

// Meeus (7.1): the Julian day of a Gregorian calendar date in UT.
double julian_day(int year, int month, double day)
{
    if (month < 3) {
        year -= 1;
        month += 12;
    }
    double jd = std::trunc(365.25 * (year + 4716.0)) + std::trunc(30.6001 * (month + 1)) + day -
                1524.5;
    if (jd > 2299160.0) {
        const double a = std::trunc(year / 100.0);
        jd += 2.0 - a + std::trunc(a / 4.0);
    }
    return jd;
}

}  // namespace

int position(const facetcu_solar_input& in, double* zenith, double* azimuth)
{
    if (const int err = validate(in)) return err;
    const double day = in.day + (in.hour - in.timezone + (in.minute + in.second / 60.0) / 60.0) /
                                    24.0;
    const double jd = julian_day(in.year, in.month, day);
    const double jde = jd + in.delta_t / 86400.0;
    const double t = (jde - 2451545.0) / 36525.0;  // ephemeris centuries from J2000
    const double tu = (jd - 2451545.0) / 36525.0;  // the same in UT

    // the sun's geometric longitude and radius vector (Meeus chapter 25)
    const double l0 = 280.46646 + 36000.76983 * t + 0.0003032 * t * t;
    const double m = 357.52911 + 35999.05029 * t - 0.0001537 * t * t;
    const double ecc = 0.016708634 - 0.000042037 * t - 0.0000001267 * t * t;
    const double c = (1.914602 - 0.004817 * t - 0.000014 * t * t) * std::sin(rad(m)) +
                     (0.019993 - 0.000101 * t) * std::sin(rad(2.0 * m)) +
                     0.000289 * std::sin(rad(3.0 * m));
    const double true_longitude = l0 + c;
    const double anomaly = m + c;
    const double r = 1.000001018 * (1.0 - ecc * ecc) / (1.0 + ecc * std::cos(rad(anomaly)));

    // nutation (Meeus chapter 22, the four main terms) and obliquity (22.2)
    const double omega = 125.04452 - 1934.136261 * t;
    const double ls = 280.4665 + 36000.7698 * t, lm = 218.3165 + 481267.8813 * t;
    const double dpsi = (-17.20 * std::sin(rad(omega)) - 1.32 * std::sin(rad(2.0 * ls)) -
                         0.23 * std::sin(rad(2.0 * lm)) + 0.21 * std::sin(rad(2.0 * omega))) /
                        3600.0;
    const double deps = (9.20 * std::cos(rad(omega)) + 0.57 * std::cos(rad(2.0 * ls)) +
                         0.10 * std::cos(rad(2.0 * lm)) - 0.09 * std::cos(rad(2.0 * omega))) /
                        3600.0;
    const double eps0 = 23.0 + 26.0 / 60.0 +
                        (21.448 - 46.8150 * t - 0.00059 * t * t + 0.001813 * t * t * t) / 3600.0;
    const double eps = eps0 + deps;

    // apparent longitude: nutation and aberration; right ascension, declination
    const double lambda = true_longitude + dpsi - 20.4898 / 3600.0 / r;
    const double alpha = deg(std::atan2(std::cos(rad(eps)) * std::sin(rad(lambda)),
                                        std::cos(rad(lambda))));
    const double delta = deg(std::asin(std::sin(rad(eps)) * std::sin(rad(lambda))));

    // apparent sidereal time at Greenwich (Meeus 12.4 plus the nutation in
    // right ascension) and the local hour angle
    const double theta0 = 280.46061837 + 360.98564736629 * (jd - 2451545.0) +
                          0.000387933 * tu * tu - tu * tu * tu / 38710000.0;
    const double nu = theta0 + dpsi * std::cos(rad(eps));
    const double h = wrap360(nu + in.longitude - alpha);

    // topocentric place (Meeus chapter 40): the observer's geocentric
    // position from latitude and elevation, the sun's parallax
    const double phi = rad(in.latitude);
    const double xi = rad(8.794 / 3600.0 / r);
    const double u = std::atan(0.99664719 * std::tan(phi));
    const double x = std::cos(u) + in.elevation / 6378140.0 * std::cos(phi);
    const double y = 0.99664719 * std::sin(u) + in.elevation / 6378140.0 * std::sin(phi);
    const double hr = rad(h), dr = rad(delta);
    const double dalpha = std::atan2(-x * std::sin(xi) * std::sin(hr),
                                     std::cos(dr) - x * std::sin(xi) * std::cos(hr));
    const double delta_t = std::atan2((std::sin(dr) - y * std::sin(xi)) * std::cos(dalpha),
                                      std::cos(dr) - x * std::sin(xi) * std::cos(hr));
    const double ht = hr - dalpha;

    // elevation with SPA's refraction, zenith, azimuth from north eastward
    const double e0 = deg(std::asin(std::sin(phi) * std::sin(delta_t) +
                                    std::cos(phi) * std::cos(delta_t) * std::cos(ht)));
    double de = 0.0;
    if (e0 >= -(kSunRadius + in.atmos_refract))
        de = (in.pressure / 1010.0) * (283.0 / (273.0 + in.temperature)) * 1.02 /
             (60.0 * std::tan(rad(e0 + 10.3 / (e0 + 5.11))));
    *zenith = 90.0 - (e0 + de);
    const double gamma = deg(std::atan2(std::sin(ht), std::cos(ht) * std::sin(phi) -
                                                          std::tan(delta_t) * std::cos(phi)));
    *azimuth = wrap360(gamma + 180.0);
    return 0;
}

// updateSolarPosition (facetrtcore.cpp:3290-3327) on one meteorology row.
int faceteb_sun(float julian_time, float latitude, float longitude, float pressure,
                float air_temperature, float* zenith, float* azimuth)
{
    constexpr int kYear = 2019;
    const int doy = static_cast<int>(std::floor(julian_time));
    // Utils::calculateMonthAndDay: months of 2019 (not a leap year); a day
    // beyond the year stays in December and fails SPA's day check
    static const int days_in_month[12] = {31, 28, 31, 30, 31, 30, 31, 31, 30, 31, 30, 31};
    int month = 0, day = doy;
    while (month < 11 && day > days_in_month[month]) day -= days_in_month[month++];
    const double fraction = static_cast<double>(julian_time) - doy;
    const double local_hours = fraction * 24.0;
    const int hour = static_cast<int>(std::floor(local_hours));
    const int minute = static_cast<int>(std::floor((local_hours - static_cast<double>(hour)) * 60.0));
    facetcu_solar_input in{};
    in.year = kYear;
    in.month = month + 1;
    in.day = day;
    in.hour = std::clamp(hour, 0, 23);
    in.minute = std::clamp(minute, 0, 59);
    in.second = 0;
    in.timezone = 8.0;
    // Utils::calculateDeltaT(2019, month): its decimal year truncates to
    // 2019 in every month, in the 2005-2050 polynomial
    const int years = kYear - 2000;
    in.delta_t = 62.92 + 0.32217 * years + 0.005589 * std::pow(years, 2);
    in.longitude = longitude;
    in.latitude = latitude;
    in.elevation = 100.0;
    in.pressure = std::max(100.0f, pressure);
    in.temperature = air_temperature;
    in.atmos_refract = 0.5667;
    double z = 0.0, a = 0.0;
    if (position(in, &z, &a) != 0) return 1;
    *zenith = static_cast<float>(z);
    *azimuth = static_cast<float>(a);
    return 0;
}

}  // namespace solar
}  // namespace facetcu

extern "C" {

int facetcu_solar_position(const facetcu_solar_input* input, double* zenith, double* azimuth,
                           int32_t* spa_error)
{
    facetcu_set_host_error("");
    if (!input || !zenith || !azimuth) {
        facetcu_set_host_error("input, zenith and azimuth are required");
        return FACETCU_INVALID_ARGUMENT;
    }
    const int err = facetcu::solar::position(*input, zenith, azimuth);
    if (spa_error) *spa_error = err;
    if (err) {
        facetcu_set_host_error("solar position: input out of range (SPA error code " +
                               std::to_string(err) + ")");
        return FACETCU_INVALID_ARGUMENT;
    }
    return FACETCU_OK;
}

int facetcu_faceteb_sun(float julian_time, float latitude, float longitude, float pressure,
                        float air_temperature, float* zenith, float* azimuth)
{
    facetcu_set_host_error("");
    if (!zenith || !azimuth) {
        facetcu_set_host_error("zenith and azimuth are required");
        return FACETCU_INVALID_ARGUMENT;
    }
    if (facetcu::solar::faceteb_sun(julian_time, latitude, longitude, pressure, air_temperature,
                                    zenith, azimuth) != 0) {
        facetcu_set_host_error("FacetEB solar-position calculation failed");
        return FACETCU_RUNTIME_ERROR;
    }
    return FACETCU_OK;
}

}  // extern "C"
