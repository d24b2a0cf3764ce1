/*
 * TEST INFRASTRUCTURE ONLY -- stand-in for <boost/version.hpp>: the version the reference's
 * utilities.hpp:176-184 tests for its assume-aligned workaround (any release from 1.61 on).
 */
#pragma once
#define BOOST_VERSION 106600
