/* TEST INFRASTRUCTURE — included by the reference, nothing used. */
#pragma once
