/* Empty stand-in: the SuperDCA headers compiled by the test oracle include
 * this boost header but use nothing from it on the solve path. */
#pragma once
